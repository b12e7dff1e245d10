"""Batched persistent DPCG (fcg_batch_dpcg): every system of a batch against its own
fcg_dpcg solve (dpcg.f90's recurrence and stop test per system), mixed sizes, early
exits, determinism, the autotuner, and argument errors."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg

pytestmark = pytest.mark.gpu


def _system(N, seed, jitter=0.2, zero_rhs=False):
    m = fcg.hex_mesh(N, jitter=jitter, seed=seed)
    ctx = fcg.Context(m)
    su0 = np.zeros(m.numCells) if zero_rhs else fcg.uniform(seed, 0, m.numCells) * m.vol
    a, su = ctx.laplacian(np.full(m.numCells, -1.0), np.zeros(m.numTotal), su0)
    return ctx, a, su


def _rel(a, b):
    return np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)


SIZES = [(8, 1, 0.2), (12, 2, 0.0), (16, 3, 0.25), (10, 4, 0.1), (20, 5, 0.2)]


def test_batch_matches_single_solves_fixed_sweeps_and_converged():
    systems = [_system(N, s, j) for N, s, j in SIZES]
    ctxs = [c for c, _, _ in systems]
    a = [x for _, x, _ in systems]
    su = [x for _, _, x in systems]
    x0 = [np.zeros(c.n) for c in ctxs]
    b = fcg.Batch(ctxs)
    # fixed sweeps: only the grouping of the global sums differs from fcg_dpcg
    fi, reps = b.dpcg(a, su, x0, 0.0, 25)
    for k, (c, ak, sk) in enumerate(systems):
        ref = c.dpcg(ak, sk, x0[k], 0.0, 25)
        assert reps[k].iters == 25
        assert _rel(fi[k], ref.fi) < 1e-10
        assert reps[k].res0 == pytest.approx(ref.res0, rel=1e-13)
    # converged, each system to its own stop test; smaller systems stop earlier
    fi, reps = b.dpcg(None, su, x0, 1e-8, 5000)
    for k, (c, ak, sk) in enumerate(systems):
        ref = c.dpcg(ak, sk, x0[k], 1e-8, 5000)
        assert reps[k].converged and abs(reps[k].iters - ref.iters) <= 1
        assert reps[k].resl / reps[k].res0 < 1e-8 and reps[k].l2_rel < 1e-7
        assert _rel(fi[k], ref.fi) < 1e-7
        # the true residual of the returned solution
        res = sk - c.spmv(ak, fi[k])
        assert np.abs(res).sum() / reps[k].res0 < 1e-8
    assert len({r.iters for r in reps}) > 1
    b.close()


def test_batch_early_exit_and_determinism():
    systems = [_system(10, 7), _system(6, 8, zero_rhs=True), _system(14, 9)]
    ctxs = [c for c, _, _ in systems]
    a = [x for _, x, _ in systems]
    su = [x for _, _, x in systems]
    x0 = [np.zeros(c.n) for c in ctxs]
    b = fcg.Batch(ctxs)
    fi1, reps = b.dpcg(a, su, x0, 1e-8, 5000)
    assert reps[1].iters == 0 and reps[1].res0 == 0.0  # dpcg.f90:66-70
    assert np.all(fi1[1] == 0.0)
    assert reps[0].converged and reps[2].converged
    fi2, _ = b.dpcg(None, su, x0, 1e-8, 5000)
    for u, v in zip(fi1, fi2):
        assert np.array_equal(u, v)
    b.close()


def test_batch_autotune_and_device_arrays():
    torch = pytest.importorskip("torch")
    systems = [_system(N, s, j) for N, s, j in SIZES[:3]]
    ctxs = [c for c, _, _ in systems]
    a = [torch.from_numpy(x).cuda() for _, x, _ in systems]
    su = [torch.from_numpy(x).cuda() for _, _, x in systems]
    x0 = [torch.zeros(c.n, dtype=torch.float64, device="cuda") for c in ctxs]
    b = fcg.Batch(ctxs)
    best = b.autotune(a, su, sweeps=10)
    p = b.params
    assert best > 0 and p["slices_per_item"] in (4, 8, 16, 32, 64, 128)
    assert 1 <= p["blocks_per_sm"] <= p["max_blocks_per_sm"]
    fi, reps = b.dpcg(a, su, x0, 1e-8, 5000)
    for k, (c, ak, sk) in enumerate(systems):
        ref = c.dpcg(ak, sk, np.zeros(c.n), 1e-8, 5000)
        assert reps[k].converged
        assert _rel(fi[k].cpu().numpy(), ref.fi) < 1e-7
    # every candidate gives the same solution to rounding
    for spi, bps in ((4, 1), (128, p["max_blocks_per_sm"])):
        b.set_params(spi, bps)
        fj, _ = b.dpcg(None, su, x0, 0.0, 20)
        ref = [c.dpcg(ak, sk, np.zeros(c.n), 0.0, 20).fi for c, ak, sk in systems]
        for u, v in zip(fj, ref):
            assert _rel(u.cpu().numpy(), v) < 1e-10
    b.close()


def test_batch_argument_errors():
    c1, a1, s1 = _system(6, 1)
    with pytest.raises(fcg._lib.FcgError):
        fcg.Batch([c1, c1])  # two systems cannot share one context's solver vectors
    b = fcg.Batch([c1])
    with pytest.raises(fcg._lib.FcgError):
        b.set_params(16, b.params["max_blocks_per_sm"] + 1)
    b.close()


def test_barrier_wait_runs_out_and_device_stays_usable():
    """A CTA that never reaches the grid barrier: the others give up after the poll limit,
    the call returns FCG_ERR_TIMEOUT, and the same batch then solves normally."""
    systems = [_system(8, 1), _system(10, 2)]
    ctxs = [c for c, _, _ in systems]
    a = [x for _, x, _ in systems]
    su = [x for _, _, x in systems]
    x0 = [np.zeros(c.n) for c in ctxs]
    b = fcg.Batch(ctxs)
    b.set_wait_test(polls=4096, absent_block=0)
    with pytest.raises(fcg._lib.FcgError) as ei:
        b.dpcg(a, su, x0, 1e-8, 500)
    assert ei.value.status == fcg._lib.FCG_ERR_TIMEOUT
    b.set_wait_test(0, -1)
    fi, reps = b.dpcg(a, su, x0, 1e-8, 500)
    for k, (c, ak, sk) in enumerate(systems):
        ref = c.dpcg(ak, sk, x0[k], 1e-8, 500)
        assert reps[k].converged and _rel(fi[k], ref.fi) < 1e-7
    b.close()
