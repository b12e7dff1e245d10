"""DIC / DILU triangular sweeps in their three kernel forms against each other: one
launch per level, one launch with rows waiting on the rows they read, and (on meshes
that form a lexicographic hex block) the wavefront-tiled launch.  All use the same row
arithmetic in the same entry order, so the same bits.  And the timeout path of the
dependency waits: a row that never announces its result makes the solve return
FCG_ERR_TIMEOUT, and the context then solves normally."""
import os

import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300 import _lib
from oracle import oracle
from tests.meshes import fixture_mesh, hex_mesh, oracle_csr, poisson_system

pytestmark = pytest.mark.gpu


def _context(m, levels, tile=None):
    """A context whose solver state (created at its first solve) uses the level
    launches (levels=True or "levels"), the row-claiming one-launch sweeps ("rows") or
    the default (False: wavefront tiles on hex blocks, rows elsewhere); tile="8x8"
    selects 8 x 8 wavefront tiles instead of 16 x 8."""
    saved = {k: os.environ.get(k) for k in ("FCG_SWEEP", "FCG_WAVE_TILE")}
    mode = "levels" if levels is True else levels
    if mode:
        os.environ["FCG_SWEEP"] = mode
    else:
        os.environ.pop("FCG_SWEEP", None)
    if tile:
        os.environ["FCG_WAVE_TILE"] = tile
    else:
        os.environ.pop("FCG_WAVE_TILE", None)
    try:
        c = fcg.Context(m)
        c.set_solver_options(float(np.float32(1e-20)), True)  # creates the solver state
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return c


@pytest.mark.parametrize("name", ["hex12", "hex20", "hex33", "pitzdaily"])
def test_one_launch_sweeps_equal_level_sweeps(name):
    """hex12 is one 16 x 8 tile and a partial one (one 8 x 8 tile and partial ones in the
    8 x 8 form), hex20 and hex33 cut tiles at the block edge and have tiles that wait on
    several others; pitzDaily is not a block (no wavefront form)."""
    m = fixture_mesh("pitzdaily") if name == "pitzdaily" else hex_mesh(int(name[3:]), 0.2)
    ctxs = [_context(m, False), _context(m, False, "8x8"), _context(m, "rows"),
            _context(m, "levels")]
    mu, phi, su0 = poisson_system(m)
    a, su = ctxs[0].laplacian(mu, phi, su0)
    x0 = np.zeros(m.numCells)
    for solver in ("iccg", "bicgstab"):
        for sor, nsw in ((0.0, 30), (1e-8, 3000)):
            r = [getattr(c, solver)(a, su, x0, sor, nsw) for c in ctxs]
            for other in r[1:]:
                assert other.iters == r[0].iters and np.array_equal(other.fi, r[0].fi), (solver, sor)
                assert other.resl == r[0].resl
    for c in ctxs:
        c.close()


def test_sweep_wait_runs_out_and_device_stays_usable():
    m = hex_mesh(10, 0.2)
    c = fcg.Context(m)
    mu, phi, su0 = poisson_system(m)
    a, su = c.laplacian(mu, phi, su0)
    x0 = np.zeros(m.numCells)
    c.set_sweep_wait_test(polls=2048, absent_row=m.numCells // 2)
    with pytest.raises(_lib.FcgError) as ei:
        c.iccg(a, su, x0, 1e-8, 50)
    assert ei.value.status == _lib.FCG_ERR_TIMEOUT
    assert "dependency wait" in str(ei.value)
    c.set_sweep_wait_test(0, 0)
    r = c.iccg(a, su, x0, 1e-8, 3000)
    o = oracle.iccg(oracle_csr(m), a, su, x0.copy(), 1e-8, 3000)
    assert r.converged and abs(r.iters - o.iters) <= 1
    assert np.abs(r.fi - o.fi).max() / np.abs(o.fi).max() < 1e-8
    c.close()


@pytest.mark.parametrize("name", ["hex16", "pitzdaily"])
def test_multi_rhs_one_launch_sweeps_equal_level_sweeps(name):
    """The FP32 DILU sweeps of the multi-RHS BiCGStab in both kernel forms."""
    from freecappuccino_gb300.systems import transport_systems

    m = hex_mesh(16, 0.2) if name == "hex16" else fixture_mesh("pitzdaily")
    csr = oracle_csr(m)
    a, su, _ = transport_systems(m, (csr.ioffset, csr.ja, csr.diag, csr.slot_pn, csr.slot_np))
    out = []
    for levels in (False, True):
        c = _context(m, levels)
        old = os.environ.get("FCG_SWEEP")
        if levels:
            os.environ["FCG_SWEEP"] = "levels"  # read when the multi-RHS state is made
        try:
            out.append(c.bicgstab_multi(a, su, np.zeros_like(su), 1e-10, 2000))
        finally:
            if old is None:
                os.environ.pop("FCG_SWEEP", None)
            else:
                os.environ["FCG_SWEEP"] = old
        c.close()
    (x1, r1), (x2, r2) = out
    assert np.array_equal(x1, x2)
    assert [r.iters for r in r1] == [r.iters for r in r2]
    assert all(r.converged for r in r1)
