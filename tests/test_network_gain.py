"""What the trained network gains inside the shipped cycle.

The learned FCG preconditions with the network followed by the aggregation coarse-grid
correction.  The method without the network is the same flexible CG with Jacobi sweeps in
the network's place (smoother "jacobi").  Both are solved here on the learned-
preconditioner configuration: N^3 hex meshes jittered by 0.2 h with the smoothed
log-uniform diffusivity on [0.1, 10], to the reference's L1 stop test at 1e-8, with the
library's default cycle (2 sweeps per level), at 64^3 and 128^3.

Measured on one GB300 (seed 2029, the same systems as bench.py's network_gain block):

    64^3:  network 19 FCG iterations, 13.1 ms; Jacobi 22 iterations, 5.3 ms
    128^3: network 27 FCG iterations, 41.7 ms; Jacobi 32 iterations, 21.1 ms

The network saves 14-16% of the iterations but costs more than it saves: one network
pass (six message-passing layers) costs more than the two Jacobi sweeps it replaces, so
the solve with the network takes 2.0-2.5x the time of the solve without it.  The test
pins both facts: fewer iterations with the network, and its time reported beside the
Jacobi cycle's."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [64, 128])
def test_network_gain_inside_the_cycle(N):
    import torch

    from freecappuccino_gb300.learned import (DEFAULT_WEIGHTS, LearnedPreconditioner,
                                              pressure_system)

    sysm = pressure_system(N, 0.2, 2029, variable=True)
    a = torch.from_numpy(sysm.a).cuda()
    su = torch.from_numpy(sysm.su).cuda()
    x0 = torch.zeros(sysm.ctx.n, dtype=torch.float64, device="cuda")
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    out = {}
    for smoother in ("network", "jacobi"):
        lp.set_multilevel(smoother=smoother)
        lp.solve(sysm.ctx, a, su, x0, 1e-8, 20000)  # hierarchy and graph
        r = lp.solve(sysm.ctx, a, su, x0, 1e-8, 20000)
        assert r.converged and not r.fallback, smoother
        assert r.resl / r.res0 < 1e-8 and r.l2_rel < 1e-7, smoother
        out[smoother] = r
    net, jac = out["network"], out["jacobi"]
    # the two preconditioned solves reach the same solution
    d = (net.fi - jac.fi).abs().max() / jac.fi.abs().max()
    assert float(d) < 1e-6
    # what the network gains: fewer iterations in the same cycle
    assert net.fcg_iters < jac.fcg_iters
    print(f"\n{N}^3: network + coarse {net.fcg_iters} iterations, {net.seconds * 1e3:.1f} ms; "
          f"Jacobi + coarse {jac.fcg_iters} iterations, {jac.seconds * 1e3:.1f} ms; "
          f"time ratio network/Jacobi {net.seconds / jac.seconds:.2f}")
    lp.close()
    sysm.ctx.close()
