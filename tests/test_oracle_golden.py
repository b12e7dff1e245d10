"""Pins the CPU oracle to the reference's own golden traces.

tests/test_sparse_solvers.f90 builds two 5x5 dense-as-CSR systems and solves them with
BiCGStab(DILU) (nonsymmetric), then ICCG (DIC) and DPCG (SPD, warm-started);
tests/output.txt holds what that program printed.  The oracle replays the program
and must print the same text, character for character.
"""
import json
import os

import numpy as np

from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _f32_literals(tokens):
    # default-REAL literals: parse as float32, then promote to real(dp)
    return np.array([np.float32(t) for t in tokens], dtype=np.float32).astype(np.float64)


def _replay_test_program():
    g = json.load(open(os.path.join(GOLDEN, "sparse_solvers.json")))
    csr = oracle.CSR(np.array(g["ioffset"], np.int32), np.array(g["ja"], np.int32),
                     np.array(g["diag"], np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
    small, resmax, ns = oracle.small_test(), oracle.tol(), 100  # test copies: :36, :99
    lines = []

    def solve(kind, a, b, x):
        r = getattr(oracle, kind)(csr, a, b, x, resmax, ns, small=small, early_exit=False)
        lines.append(" " * 20 + f"res0 = {r.res0:10.3E}")
        for l, (resl, rsm) in enumerate(r.trace, start=1):
            lines.append(" " * 19 + f" iter = {l:4d} resl = {resl:10.3E} rsm = {rsm:10.3E}")
        return r.fi

    def solution(x, xa):
        lines.append(" ")
        lines.append(" " * 19 + "Solution: " + " " * 5 + "Analytic solution:")
        for xi, xai in zip(x, xa):
            lines.append(" " * 19 + f"{xi:5.2f}" + " " * 10 + f"{xai:5.2f}")

    a1, b1, xa1 = (_f32_literals(g["test1"][k]) for k in ("a", "b", "xa"))
    lines += [" ", " Test 1 - Real nonsymmetric 5x5 system.", " ", " "]
    lines.append(" " * 19 + " The ILU(0) preconditioned BiCGStab solver:")
    x = solve("bicgstab", a1, b1, np.zeros(5))  # x is never set; the trace shows it was 0
    solution(x, xa1)

    a2, b2, xa2 = (_f32_literals(g["test2"][k]) for k in ("a", "b", "xa"))
    lines += [" ", " Test 2 - symmetric positive definite 5x5 system.", " ", " "]
    lines.append(" " * 19 + " The Incomplete Cholesky preconditioned CG solver:")
    x = solve("iccg", a2, b2, x)  # warm start from test 1's solution
    solution(x, xa2)
    lines += [" "]
    lines.append(" " * 19 + " The Diagonally preconditioned CG solver:")
    x = solve("dpcg", a2, b2, x)  # warm start from ICCG's solution
    solution(x, xa2)
    return lines


def test_oracle_reproduces_reference_output_txt():
    expected = open(os.path.join(GOLDEN, "sparse_solvers_output.txt")).read().splitlines()
    got = _replay_test_program()
    assert len(got) == len(expected)
    for i, (e, o) in enumerate(zip(expected, got)):
        assert e.rstrip() == o.rstrip(), f"line {i + 1}:\n expected {e!r}\n got      {o!r}"


def test_iteration_counts_match_published_table():
    lines = _replay_test_program()
    iters = [sum(1 for l in blk.splitlines() if "iter =" in l) for blk in
             ("\n".join(lines).split("solver:")[1:])]
    assert iters == [6, 5, 5]
