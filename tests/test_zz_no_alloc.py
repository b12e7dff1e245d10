"""fcg_dpcg_noalloc: the DPCG entry point for callers that cannot allocate device memory.

Some callers own all of their GPU memory (a host code that reserves the whole device
for its own pool at start-up, or a loop that must not allocate after initialisation).
They hold the matrix and vectors on the device already and cannot let the library
cudaMalloc work space, so fcg_dpcg_noalloc takes only device arrays and keeps its work
vectors in a fixed-size array inside the library.  This test calls it through the C ABI
twice in a row and checks each result against the context-based fcg_dpcg on the same
system, within the tolerance the other solver tests use, and checks that systems beyond
its size limit are refused.  The file sorts last so that a run stopping at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300 import _lib

pytestmark = pytest.mark.gpu


def _system(N):
    m = fcg.hex_mesh(N, jitter=0.2, seed=5)
    ctx = fcg.Context(m)
    mu = np.full(m.numCells, -1.0)
    su0 = fcg.uniform(5, 0, m.numCells) * m.vol
    a, su = ctx.laplacian(mu, np.zeros(m.numTotal), su0)
    io, ja, dg, _, _ = ctx.create_csr()
    return m, ctx, a, su, io, ja, dg


def _noalloc(torch, io, ja, dg, a, su, sor, nsw, fi0=None, stream=None):
    lib = _lib.load()
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    tio, tja, tdg, ta, tsu = d(io), d(ja), d(dg), d(a), d(su)
    fi = torch.zeros(len(dg), dtype=torch.float64, device="cuda") if fi0 is None else d(fi0)
    res = torch.empty_like(fi)
    resor = C.c_double(float("nan"))
    rep = _lib.SolveReport()
    torch.cuda.synchronize()
    rc = lib.fcg_dpcg_noalloc(len(dg), tio.data_ptr(), tja.data_ptr(), tdg.data_ptr(),
                              ta.data_ptr(), tsu.data_ptr(), fi.data_ptr(), res.data_ptr(),
                              float(sor), int(nsw), C.byref(resor), C.byref(rep),
                              None if stream is None else C.c_void_p(stream.cuda_stream))
    return rc, fi.cpu().numpy(), res.cpu().numpy(), rep, resor.value


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("N", [16, 48])
def test_noalloc_matches_dpcg_twice(N):
    torch = pytest.importorskip("torch")
    m, ctx, a, su, io, ja, dg = _system(N)
    # fixed number of sweeps: only the order of the global sums differs
    ref = ctx.dpcg(a, su, np.zeros(m.numCells), 0.0, 30)
    conv = ctx.dpcg(a, su, np.zeros(m.numCells), 1e-8, 5000)
    for _ in range(2):  # the second call must not see what the first left behind
        rc, fi, res, rep, resor = _noalloc(torch, io, ja, dg, a, su, 0.0, 30)
        assert rc == _lib.FCG_OK
        assert rep.iters == 30
        assert rel(fi, ref.fi) < 1e-10
        assert np.abs(res - ref.res).max() < 1e-10 * np.abs(su).max()
        assert resor == pytest.approx(ref.resor, rel=1e-13)
        rc, fi, res, rep, _ = _noalloc(torch, io, ja, dg, a, su, 1e-8, 5000)
        assert rc == _lib.FCG_OK and rep.converged
        assert abs(rep.iters - conv.iters) <= 1
        if rep.iters == conv.iters:
            assert rel(fi, conv.fi) < 1e-10
        assert rep.l2_rel < 1e-6
    ctx.close()


def test_noalloc_rejects_oversize_and_host_arrays():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    big = _lib.FCG_ERR_ARG
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    i = torch.ones(8, dtype=torch.int32, device="cuda")
    p = lambda t: t.data_ptr()
    # beyond the fixed work array: refused before any launch
    rc = lib.fcg_dpcg_noalloc(262144 + 1, p(i), p(i), p(i), p(x), p(x), p(x), p(x), 1e-8, 10,
                              None, None, None)
    assert rc == big
    # host arrays would need staging memory: refused
    h = np.zeros(8)
    rc = lib.fcg_dpcg_noalloc(4, p(i), p(i), p(i), h.ctypes.data, p(x), p(x), p(x), 1e-8, 10,
                              None, None, None)
    assert rc == big


def test_noalloc_allocates_nothing_after_the_first_call():
    """The first call on a device loads the code and the work array (lazy module
    loading); every later call leaves the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    m, ctx, a, su, io, ja, dg = _system(16)
    lib = _lib.load()
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    tio, tja, tdg, ta, tsu = d(io), d(ja), d(dg), d(a), d(su)
    fi = torch.zeros(len(dg), dtype=torch.float64, device="cuda")
    res = torch.empty_like(fi)
    rep = _lib.SolveReport()
    args = (len(dg), tio.data_ptr(), tja.data_ptr(), tdg.data_ptr(), ta.data_ptr(),
            tsu.data_ptr(), fi.data_ptr(), res.data_ptr(), 1e-8, 500, None, C.byref(rep), None)
    torch.cuda.synchronize()
    assert lib.fcg_dpcg_noalloc(*args) == _lib.FCG_OK  # set-up call
    free0, _ = torch.cuda.mem_get_info()
    fi.zero_()
    torch.cuda.synchronize()
    assert lib.fcg_dpcg_noalloc(*args) == _lib.FCG_OK
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert rep.converged
    ctx.close()


def test_noalloc_zero_residual_and_side_stream():
    """su = A fi: res0 = 0 < tol, no sweep and resor untouched (dpcg.f90:66-70); and the
    same solve on a non-default stream as on the legacy stream."""
    torch = pytest.importorskip("torch")
    from oracle import oracle

    m, ctx, a, su, io, ja, dg = _system(12)
    x = 1e-3 * fcg.uniform(6, 1, m.numCells)  # small: rounding of A x stays far below tol
    csr = oracle.create_csr(m.numCells, m.owner, m.neighbour)
    b = oracle.spmv(csr, a, x)
    rc, fi, res, rep, resor = _noalloc(torch, io, ja, dg, a, b, 1e-8, 100, fi0=x)
    assert rc == _lib.FCG_OK
    assert rep.iters == 0 and np.isnan(resor)
    assert np.array_equal(fi, x)
    s = torch.cuda.Stream()
    rc0, fi0, _, rep0, _ = _noalloc(torch, io, ja, dg, a, su, 0.0, 20)
    rc1, fi1, _, rep1, _ = _noalloc(torch, io, ja, dg, a, su, 0.0, 20, stream=s)
    assert rc0 == rc1 == _lib.FCG_OK and rep0.iters == rep1.iters == 20
    assert np.array_equal(fi0, fi1)  # same launches, same order of sums
    ctx.close()
