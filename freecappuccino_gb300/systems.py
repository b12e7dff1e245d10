"""Synthetic inputs of the benchmark configurations: flow fields of the pressure step
and the linear systems of the multi-RHS configuration.

``transport_systems`` builds the five convection-diffusion systems of the multi-RHS
configuration on a mesh: momentum u, v, w (one set of off-diagonals, as calcuvw.f90
builds one set for all three, :157-185) plus k and epsilon (own diffusivities).  It is
an input generator, not a restatement of calcuvw: the convecting velocity is the curl
of three seeded Fourier modes, so it is divergence-free; faces use the upwind/central
blend of the reference's deferred-correction scheme with gds = 0.5 written implicitly;
diffusion uses the laplacian's |S|^2 / (S.d) (fvm_laplacian.f90:214); implicit Euler
with the time step set by max Courant = 1 adds vol/dt to the diagonal.  Walls are
Dirichlet for diffusion (fvm_laplacian.f90:140-154); no flux crosses any boundary.
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh, uniform


def flow_fields(m: Mesh, seed: int = 3):
    """Seeded flow fields of the pressure step (calcp): u, v, w, p and den of numTotal
    length (U(-1,1), den 1 +- 0.2), gradients (numCells, 3) U(-1,1), and
    ap* = (1 +- 0.1) / vol."""
    n, nt = m.numCells, m.numTotal
    u = uniform(seed, 1, nt)
    v = uniform(seed, 2, nt)
    w = uniform(seed, 3, nt)
    p = uniform(seed, 4, nt)
    g = [uniform(seed, 10 + k, 3 * n).reshape(n, 3) for k in range(4)]
    ap = [1.0 / m.vol * (1.0 + 0.1 * uniform(seed, 20 + k, n)) for k in range(3)]
    den = 1.0 + 0.2 * uniform(seed, 30, nt)
    return dict(u=u, v=v, w=w, p=p, dUdxi=g[0], dVdxi=g[1], dWdxi=g[2], dPdxi=g[3],
                apu=ap[0], apv=ap[1], apw=ap[2], den=den)


def fourier_velocity(x, y, z, seed: int, modes: int = 3):
    """u = curl(psi), psi = sum_m cos-modes: u = sum_m cos(k_m.x + phi_m) (k_m x e_m),
    scaled to unit peak amplitude of the sum of mode magnitudes."""
    u = np.zeros((len(x), 3))
    amp = 0.0
    for m in range(modes):
        r = uniform(seed, 7000 + m, 8, 0.0, 1.0)
        k = 2 * np.pi * np.floor(1 + 3 * r[:3])  # wave numbers 1..3 per axis
        e = r[3:6] - 0.5
        e /= np.linalg.norm(e)
        phase = 2 * np.pi * r[6]
        c = np.cross(k, e)
        u += np.cos(k[0] * x + k[1] * y + k[2] * z + phase)[:, None] * c[None, :]
        amp += np.linalg.norm(c)
    return u / amp


def transport_systems(m: Mesh, csr, seed: int = 1, nu: float = 1e-3, gds: float = 0.5,
                      courant: float = 1.0, nsys: int = 5):
    """Returns (a[nsys, nnz], su[nsys, n], dt): CSR values (1-based pattern `csr` =
    (ioffset, ja, diag, slot_pn, slot_np)) and right-hand sides U(-1,1)*vol."""
    io, ja, dg, spn, snp = csr
    n, nin = m.numCells, m.numInnerFaces
    P = m.owner[:nin] - 1
    N = m.neighbour - 1
    u = fourier_velocity(m.xf[:nin], m.yf[:nin], m.zf[:nin], seed)
    F = u[:, 0] * m.arx[:nin] + u[:, 1] * m.ary[:nin] + u[:, 2] * m.arz[:nin]
    lam = m.facint
    dx = m.xc[N] - m.xc[P]
    dy = m.yc[N] - m.yc[P]
    dz = m.zc[N] - m.zc[P]
    s2 = m.arx[:nin] ** 2 + m.ary[:nin] ** 2 + m.arz[:nin] ** 2
    smdpn = s2 / (m.arx[:nin] * dx + m.ary[:nin] * dy + m.arz[:nin] * dz)
    # time step: max over cells of dt/(2 vol) * sum |F| = courant
    flux_sum = np.zeros(n)
    np.add.at(flux_sum, P, np.abs(F))
    np.add.at(flux_sum, N, np.abs(F))
    dt = courant / np.max(flux_sum / (2 * m.vol))
    # wall faces (Dirichlet diffusion)
    nw, w0 = m.counts.get("nwal", 0), m.starts.get("iWallFacesStart", 0)
    wf = np.arange(w0, w0 + nw)
    wc = m.owner[wf] - 1
    are = np.sqrt(m.arx[wf] ** 2 + m.ary[wf] ** 2 + m.arz[wf] ** 2)
    dpw = np.sqrt((m.xc[wc] - m.xf[wf]) ** 2 + (m.yc[wc] - m.yf[wf]) ** 2 + (m.zc[wc] - m.zf[wf]) ** 2)
    extra_diff = [0.0, 0.0, 0.0, 1e-3, 2e-3]
    sigma = [0.0, 0.1, 0.2, 0.3, 0.5]
    a = np.zeros((nsys, len(ja)))
    su = np.zeros((nsys, n))
    up_in_p = np.maximum(-F, 0.0)   # inflow into P through the face
    up_in_n = np.maximum(F, 0.0)    # inflow into N
    for k in range(nsys):
        g = nu + extra_diff[k % 5]
        D = g * smdpn
        a_pn = -D - (1 - gds) * up_in_p + gds * F * lam
        a_np = -D - (1 - gds) * up_in_n - gds * F * (1 - lam)
        dP = D + (1 - gds) * up_in_n + gds * F * (1 - lam)
        dN = D + (1 - gds) * up_in_p - gds * F * lam
        diag = m.vol / dt * (1 + sigma[k % 5])
        np.add.at(diag, P, dP)
        np.add.at(diag, N, dN)
        np.add.at(diag, wc, g * are / dpw)
        a[k, spn - 1] = a_pn
        a[k, snp - 1] = a_np
        a[k, dg - 1] = diag
        su[k] = uniform(seed, 100 + k, n) * m.vol
    return a, su, dt
