"""Learned preconditioner and flexible CG (learned.cu).

CPU: the numpy oracle's gradient against central finite differences of its own FP64
forward, its BF16 rounding against torch's, the parameter count against the header.
GPU: features, forward, loss and gradient, and one Adam step of the CUDA kernels
against the oracle on the same inputs; checkpoint round trip; the flexible CG with the
network converges to the reference's stop test, falls back to DPCG when it stalls, and
a briefly trained network needs fewer iterations than the untrained one."""
import os
import re

import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import learned_oracle as lo
from oracle import oracle

from tests.meshes import oracle_csr, oracle_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_system(N, seed=3, variable=True):
    """Pressure system on an N^3 jittered mesh assembled by the C oracle."""
    from freecappuccino_gb300.learned import diffusivity_field

    m = fcg.hex_mesh(N, jitter=0.2, seed=seed)
    om, csr = oracle_mesh(m), oracle_csr(m)
    gam = diffusivity_field(m, seed) if variable else np.ones(m.numCells)
    su0 = fcg.uniform(seed, 0, m.numCells) * m.vol
    a, su = oracle.laplacian(om, csr, -gam, np.zeros(m.numTotal), su0)
    return m, csr, a, su


def _random_weights(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    W_in = rng.uniform(-1, 1, (lo.C, lo.F)) / np.sqrt(lo.F)
    b_in = rng.uniform(-0.2, 0.2, lo.C)
    layers = [(rng.uniform(-1, 1, (lo.C, 2 * lo.C)) * scale / np.sqrt(2 * lo.C),
               rng.uniform(-0.2, 0.2, lo.C)) for _ in range(lo.L)]
    w_out = rng.uniform(-1, 1, lo.C) / np.sqrt(lo.C)
    return lo.pack(W_in, b_in, layers, w_out, 0.05).astype(np.float32)


# ----------------------------------------------------------------------------- CPU
def test_header_parameter_count():
    txt = open(os.path.join(ROOT, "include", "fcgpu.h")).read()
    assert int(re.search(r"#define FCG_LP_PARAMS (\d+)", txt).group(1)) == lo.P
    assert int(re.search(r"#define FCG_LP_WIDTH (\d+)", txt).group(1)) == lo.C
    assert int(re.search(r"#define FCG_LP_LAYERS (\d+)", txt).group(1)) == lo.L


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(20000) * 10.0 ** rng.integers(-6, 6, 20000),
                        [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 65504.0]])
    ref = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(lo.bf16(x), ref)


@pytest.mark.parametrize("kind", ["energy", "residual", "cycle"])
def test_oracle_gradient_matches_finite_differences(kind):
    m, csr, a, su = _oracle_system(4)
    A = lo.ScaledMatrix(csr.ioffset, csr.ja, csr.diag, a)
    feat = lo.features(m, A.s)
    rng = np.random.default_rng(1)
    r = rng.standard_normal(m.numCells)
    e = rng.standard_normal(m.numCells)
    w = _random_weights(2, scale=3.0).astype(np.float64)
    correct = None
    if kind == "cycle":  # the coarse-grid correction on the same Ahat, in FP64
        from oracle import multilevel_oracle as mo

        fine = (np.asarray(csr.ioffset) - 1, np.asarray(csr.ja) - 1, A.val)
        levels = mo.build_levels(*fine)
        assert levels
        correct = mo.Cycle(fine, levels, mo.level_values(levels, fine, f32=False)).correct
    loss, g = lo.loss_grad(A, feat, r, e, w, emulate=False, kind=kind, correct=correct)
    idx = rng.choice(lo.P, 80, replace=False)
    idx = np.concatenate([idx, [lo.P - 1, 0, lo.C * lo.F]])  # b_out, W_in, b_in
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (lo.loss_grad(A, feat, r, e, wp, emulate=False, kind=kind, correct=correct)[0] -
              lo.loss_grad(A, feat, r, e, wm, emulate=False, kind=kind, correct=correct)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-7, (i, fd, g[i])


def test_oracle_features_of_uniform_cube_are_zero():
    m = fcg.hex_mesh(6, jitter=0.0, seed=1)
    om, csr = oracle_mesh(m), oracle_csr(m)
    a, _ = oracle.laplacian(om, csr, -np.ones(m.numCells), np.zeros(m.numTotal),
                            np.zeros(m.numCells))
    A = lo.ScaledMatrix(csr.ioffset, csr.ja, csr.diag, a)
    f = lo.features(m, A.s)
    # unit diffusivity on cubes: vol and face sums exactly at their reference values; the
    # diagonal is 6h in cells with no boundary face
    assert np.abs(f[:, 2:]).max() < 1e-6
    nbf = np.bincount(m.owner[m.numInnerFaces:m.numFaces] - 1, minlength=m.numCells)
    assert (nbf == 0).sum() == 4 ** 3
    assert np.abs(f[nbf == 0, 1]).max() < 1e-6
    assert np.abs(f[nbf > 0, 1]).max() > 0.1


def test_training_shard_round_trip(tmp_path):
    from freecappuccino_gb300.learned import load_pairs, save_pairs

    rng = np.random.default_rng(4)
    pairs = [(rng.standard_normal(50).astype(np.float32), rng.standard_normal(50).astype(np.float32))
             for _ in range(3)]
    path = str(tmp_path / "shard.npz")
    save_pairs(path, pairs, {"N": 64, "seed": 7, "jitter": 0.125})
    back, meta = load_pairs(path)
    assert meta == {"N": 64, "seed": 7, "jitter": 0.125}
    for (r0, e0), (r1, e1) in zip(pairs, back):
        assert np.array_equal(r0, r1) and np.array_equal(e0, e1)


# ----------------------------------------------------------------------------- GPU
def _gpu_system(N, seed=3, variable=True):
    from freecappuccino_gb300.learned import pressure_system

    return pressure_system(N, 0.2, seed, variable=variable)


def _pair(sysm, k):
    from freecappuccino_gb300.learned import dpcg_pairs

    return dpcg_pairs(sysm, [k])[0]


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.gpu
def test_features_match_oracle():
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(12)
    lp = LearnedPreconditioner(seed=1)
    lp.set_matrix(sysm.ctx, sysm.a)
    f = lp.features(sysm.ctx)
    ref = lo.features(sysm.mesh, sysm.scale)
    assert np.abs(f[:, 1:] - ref[:, 1:]).max() < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("N", [10, 24])
def test_forward_matches_oracle(N):
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(N)
    io, ja, dg, _, _ = sysm.ctx.create_csr()
    A = lo.ScaledMatrix(io, ja, dg, sysm.a)
    lp = LearnedPreconditioner(seed=1)
    w = _random_weights(4, scale=2.0)
    lp.weights = w
    lp.set_matrix(sysm.ctx, sysm.a)
    r, _ = _pair(sysm, 3)
    z = lp.apply(sysm.ctx, r)
    feat = lo.features(sysm.mesh, sysm.scale)
    zr, _ = lo.forward(A, feat, r, w, emulate=True)
    z64, _ = lo.forward(A, feat, r, w, emulate=False)
    # BF16 emulation: only accumulation order differs (FP32 vs FP64), which flips a
    # BF16 rounding now and then
    assert _rel(z, zr) < 5e-3
    # and the whole BF16 error against the FP64 network stays at the BF16 level
    assert _rel(z, z64) < 5e-2
    # positive homogeneity: N(2r) = 2 N(r) exactly up to the rms rounding
    z2 = lp.apply(sysm.ctx, 2 * r)
    assert _rel(z2, 2 * z) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["energy", "residual"])
def test_loss_gradient_matches_oracle(kind):
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(14)
    io, ja, dg, _, _ = sysm.ctx.create_csr()
    A = lo.ScaledMatrix(io, ja, dg, sysm.a)
    lp = LearnedPreconditioner(seed=1)
    lp.set_loss(kind)
    w = _random_weights(5, scale=2.0)
    lp.weights = w
    lp.set_matrix(sysm.ctx, sysm.a)
    r, e = _pair(sysm, 5)
    loss, g = lp.loss_grad(sysm.ctx, r, e)
    feat = lo.features(sysm.mesh, sysm.scale)
    lr_, gr = lo.loss_grad(A, feat, r, e, w, emulate=True, kind=kind)
    assert loss == pytest.approx(lr_, rel=2e-3)
    # per parameter group: embedding, each layer, output
    bounds = [0, lo.C * lo.F + lo.C] + [lo.C * lo.F + lo.C + (l + 1) * lo.LAYER
                                         for l in range(lo.L)] + [lo.P]
    for b0, b1 in zip(bounds[:-1], bounds[1:]):
        assert _rel(g[b0:b1], gr[b0:b1]) < 2e-2, (b0, b1)
    # deterministic: the same call gives the same bits
    loss2, g2 = lp.loss_grad(sysm.ctx, r, e)
    assert loss2 == loss and np.array_equal(g, g2)


@pytest.mark.gpu
def test_adam_step_matches_oracle_and_checkpoint_round_trip(tmp_path):
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(10)
    lp = LearnedPreconditioner(seed=3)
    lp.set_matrix(sysm.ctx, sysm.a)
    r, e = _pair(sysm, 2)
    w0 = lp.weights
    m = np.zeros(lo.P, np.float32)
    v = np.zeros(lo.P, np.float32)
    for step in (1, 2, 3):
        _, g = lp.loss_grad(sysm.ctx, r, e)
        lp.train_step(sysm.ctx, r, e, 1e-3)
        w0, m, v = lo.adam(w0, m, v, g, 1e-3, step)
        assert np.abs(lp.weights - w0).max() < 1e-6
    path = str(tmp_path / "lp.fcglp")
    lp.save(path)
    lp2 = LearnedPreconditioner(seed=99, path=path)
    assert np.array_equal(lp2.weights, lp.weights)
    lp2.set_matrix(sysm.ctx, sysm.a)
    lp.set_matrix(sysm.ctx, sysm.a)
    a1 = lp.train_step(sysm.ctx, r, e, 1e-3)
    a2 = lp2.train_step(sysm.ctx, r, e, 1e-3)
    assert a1 == a2 and np.array_equal(lp.weights, lp2.weights)  # Adam state restored too
    with open(path, "r+b") as f:
        f.write(b"XXXX")
    with pytest.raises(fcg._lib.FcgError):
        lp2.load(path)


@pytest.mark.gpu
def test_fcg_converges_and_matches_dpcg():
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(20, variable=False)
    lp = LearnedPreconditioner(seed=1)
    x0 = np.zeros(sysm.ctx.n)
    ref = sysm.ctx.dpcg(sysm.a, sysm.su, x0, 1e-12, 20000)
    r = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 20000)
    assert r.converged and r.resl / r.res0 < 1e-8
    assert r.l2_rel < 1e-7
    assert _rel(r.fi, ref.fi) < 1e-6
    # the fcg's own true residual agrees with a separate FP64 matvec
    res = sysm.su - sysm.ctx.spmv(sysm.a, r.fi)
    assert np.abs(res).sum() / r.res0 < 1e-8


@pytest.mark.gpu
def test_fcg_stall_falls_back_to_dpcg():
    from freecappuccino_gb300.learned import LearnedPreconditioner

    sysm = _gpu_system(16)
    lp = LearnedPreconditioner(seed=1)
    lp.set_multilevel(enabled=False)  # the network alone
    lp.set_fcg_options(directions=2, ru_every=5, stall_window=10, stall_factor=1e-9)
    x0 = np.zeros(sysm.ctx.n)
    r = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 5000)
    assert r.fallback and r.converged
    assert r.fcg_iters >= 10 and r.iters > r.fcg_iters
    assert r.resl / r.res0 < 1e-8 and r.l2_rel < 1e-7
    # a budget the FCG uses up is not topped up
    lp.set_fcg_options()
    r2 = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 3)
    assert not r2.converged and r2.iters == 3 and not r2.fallback


@pytest.mark.gpu
def test_training_reduces_loss_and_fcg_iterations():
    """What a briefly trained network gains over the untrained one: trained on DPCG
    iterates of two 16^3 systems, tested on a third (other seed)."""
    from freecappuccino_gb300.learned import LearnedPreconditioner, dpcg_pairs, train

    systems = [_gpu_system(16, seed=s) for s in (11, 12)]
    pairs = []
    for s in systems:
        conv = s.ctx.dpcg(s.a, s.su, np.zeros(s.ctx.n), 1e-8, 5000).iters
        pairs.append(dpcg_pairs(s, np.linspace(0, conv, 24).astype(int)))
    lp = LearnedPreconditioner(seed=5)
    lp.set_multilevel(enabled=False)  # the network alone
    test = _gpu_system(16, seed=13)
    x0 = np.zeros(test.ctx.n)
    before = lp.solve(test.ctx, test.a, test.su, x0, 1e-8, 5000)
    losses = train(lp, systems, pairs, steps=600, lr=2e-3, seed=0)
    assert losses[-100:].mean() < 0.7 * losses[:50].mean()
    after = lp.solve(test.ctx, test.a, test.su, x0, 1e-8, 5000)
    dpcg = test.ctx.dpcg(test.a, test.su, x0, 1e-8, 5000)
    assert after.converged and not after.fallback
    assert after.fcg_iters < before.fcg_iters
    assert after.fcg_iters < dpcg.iters
    print(f"\n16^3 held-out: DPCG {dpcg.iters} sweeps; FCG untrained {before.fcg_iters} "
          f"(fallback {before.fallback}), trained 600 steps {after.fcg_iters}")


@pytest.mark.gpu
def test_shipped_weights_beat_jacobi_in_iterations():
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner

    if not os.path.exists(DEFAULT_WEIGHTS):
        pytest.skip("no shipped checkpoint")
    sysm = _gpu_system(32, seed=21, variable=False)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_multilevel(enabled=False)  # the network alone
    x0 = np.zeros(sysm.ctx.n)
    r = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 20000)
    d = sysm.ctx.dpcg(sysm.a, sysm.su, x0, 1e-8, 20000)
    assert r.converged and not r.fallback and r.l2_rel < 1e-7
    assert r.fcg_iters < d.iters
    print(f"\n32^3 jittered: DPCG {d.iters} sweeps, learned FCG {r.fcg_iters} iterations")
