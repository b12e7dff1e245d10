"""The plane-staged layer of the learned preconditioner (learned_hex.cu) against the
sliced gather form (k_lp_layer in learned.cu).

On a mesh whose cells form a lexicographic hex block the network's layers run as
TMA-staged planes; on every other mesh they run as the gather over the sliced pattern.
Both sum each cell's neighbour terms in the CSR column order with the same fused
multiply-adds and share the tensor-core tile code, so the network's output, and every
solve it preconditions, must be bit-identical whichever form runs.  The sizes cover
tiles cut by the block edge (N = 5, 17), a last chunk of one plane (N = 33) and several
chunks (N = 40).  FCG_LP_LAYER=gather selects the gather form for the comparison."""
import os

import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner, pressure_system
from tests.meshes import fixture_mesh

pytestmark = pytest.mark.gpu


class gather_form:
    def __enter__(self):
        self.old = os.environ.get("FCG_LP_LAYER")
        os.environ["FCG_LP_LAYER"] = "gather"

    def __exit__(self, *exc):
        if self.old is None:
            os.environ.pop("FCG_LP_LAYER", None)
        else:
            os.environ["FCG_LP_LAYER"] = self.old


@pytest.mark.parametrize("N", [5, 17, 33, 40])
def test_planes_equal_gather_bit_for_bit(N):
    sysm = pressure_system(N, 0.2, 3, variable=True)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_matrix(sysm.ctx, sysm.a)
    assert lp.layer_form(sysm.ctx) == {"form": "planes", "dims": (N, N, N)}
    r = fcg.uniform(N, 9, sysm.ctx.n, -1.0, 1.0).astype(np.float32)
    z_planes = lp.apply(sysm.ctx, r)
    with gather_form():
        assert lp.layer_form(sysm.ctx)["form"] == "gather"
        z_gather = lp.apply(sysm.ctx, r)
    assert np.isfinite(z_planes).all()
    assert np.array_equal(z_planes, z_gather)
    lp.close()


def test_learned_solve_identical_with_either_form():
    sysm = pressure_system(24, 0.2, 5, variable=True)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    x0 = np.zeros(sysm.ctx.n)
    r1 = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 2000)
    assert lp.layer_form(sysm.ctx)["form"] == "planes"
    with gather_form():
        r2 = lp.solve(sysm.ctx, sysm.a, sysm.su, x0, 1e-8, 2000)
    assert r1.converged and r2.converged
    assert r1.fcg_iters == r2.fcg_iters
    assert np.array_equal(r1.fi, r2.fi)
    lp.close()


def test_other_meshes_use_the_gather_form():
    """pitzDaily (unstructured) and the 20 x 20 x 1 cavity (no third direction) keep the
    gather form; a hex mesh whose boundary patches are relabelled is still a block."""
    from tests.meshes import mixed_patch_mesh

    for m, form in ((fixture_mesh("pitzdaily"), "gather"), (fixture_mesh("cavity"), "gather"),
                    (mixed_patch_mesh(8), "planes")):
        c = fcg.Context(m)
        mu = np.full(m.numCells, -1.0)
        a, _ = c.laplacian(mu, np.zeros(m.numTotal), np.zeros(m.numCells))
        lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
        lp.set_matrix(c, a)
        assert lp.layer_form(c)["form"] == form
        z = lp.apply(c, fcg.uniform(1, 2, m.numCells).astype(np.float32))
        assert np.isfinite(z).all()
        lp.close()
        c.close()


def test_tensor_memory_form_equals_mma_sync_form():
    """The plane-staged layer with its tile product on tcgen05 (accumulator in tensor
    memory, FCG_LP_HEX_MMA=tc) gives the same bits as with mma.sync."""
    sysm = pressure_system(20, 0.2, 4, variable=True)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_matrix(sysm.ctx, sysm.a)
    r = fcg.uniform(20, 3, sysm.ctx.n, -1.0, 1.0).astype(np.float32)
    z_sync = lp.apply(sysm.ctx, r)
    old = os.environ.get("FCG_LP_HEX_MMA")
    os.environ["FCG_LP_HEX_MMA"] = "tc"
    try:
        z_tc = lp.apply(sysm.ctx, r)
    finally:
        if old is None:
            os.environ.pop("FCG_LP_HEX_MMA", None)
        else:
            os.environ["FCG_LP_HEX_MMA"] = old
    assert np.array_equal(z_sync, z_tc)
    lp.close()
