"""Momentum assembly (calcuvw.f90:48-438 with facefluxuvw, sngrad, face_value and
calcPressDiv).

The CPU tests pin the C oracle against a vectorised numpy statement of the same loops.
Per-face terms are computed elementwise in the reference's operation order, and every
scatter is an ufunc.at over the interleaved (owner, neighbour) list, which applies the
terms one by one in face order. The GPU tests compare fcg_calcuvw with the oracle bit
for bit, over every face-value scheme and limiter and the time-stepping and source
options. They then solve the three systems as calcuvw does, and with one multi-RHS
call."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300 import _lib
from oracle import oracle
from tests.meshes import fixture_mesh, hex_mesh, oracle_csr, oracle_mesh, seeded_fields

F32_099 = float(np.float32(0.99))
SMALL = float(np.float32(1e-20))


def _fields(m, seed):
    f = seeded_fields(m, seed)
    n, nt, nin = m.numCells, m.numTotal, m.numInnerFaces
    f["vis"] = 1e-3 * (1.0 + 0.5 * fcg.uniform(seed, 50, nt, 0.0, 1.0))
    f["flmass"] = 0.05 * fcg.uniform(seed, 51, nin)
    f["fmi"] = -0.01 * fcg.uniform(seed, 52, m.counts.get("ninl", 0), 0.0, 1.0)
    f["fmo"] = 0.01 * fcg.uniform(seed, 53, m.counts.get("nout", 0), 0.0, 1.0)
    f["den"] = f["den"][:n].copy()
    for k, s in (("t", 54), ("uo", 55), ("vo", 56), ("wo", 57), ("uoo", 58), ("voo", 59),
                 ("woo", 60)):
        f[k] = fcg.uniform(seed, s, n) + (290.0 if k == "t" else 0.0)
    return f


def _a_in(m, seed):
    return fcg.uniform(seed, 70, m.nnz)  # whatever the previous solve left in a


OPTS = [dict(scheme=s) for s in ("cds", "cds_corrected", "central", "second_upwind", "muscl")]
OPTS += [dict(scheme="flux_limiter", limiter=lm) for lm in _lib.LIMITERS]
OPTS += [
    dict(scheme="muscl", bdf=True, btime=0.0, timestep=0.01),
    dict(scheme="muscl", bdf=True, btime=1.0, timestep=0.02, cn=True),
    dict(scheme="central", cn=True, timestep=0.05, gds=0.5),
    dict(scheme="muscl", const_mflux=True, gradPcmf=0.3, buoyancy=True, boussinesq=True,
         beta=3e-3, densit=1.2, tref=290.0, grav=(0.0, -9.81, 0.5)),
    dict(scheme="cds", buoyancy=True, boussinesq=False, densit=1.1, grav=(0.3, -9.81, 0.0),
         urf=(0.6, 0.7, 0.8)),
]


def _oracle_params(kw):
    urf = kw.get("urf", (0.7, 0.7, 0.7))
    g = kw.get("grav", (0.0, 0.0, 0.0))
    return oracle.UvwParams(
        _lib.CONV_SCHEMES[kw.get("scheme", "muscl")], _lib.LIMITERS[kw.get("limiter", "uds")],
        kw.get("gds", 1.0), kw.get("viscos", 1e-3), (oracle.C.c_double * 3)(*[1.0 / x for x in urf]),
        (oracle.C.c_double * 3)(*[1.0 - x for x in urf]), int(kw.get("bdf", False)),
        int(kw.get("cn", False)), kw.get("timestep", 1.0), kw.get("btime", 0.0),
        int(kw.get("const_mflux", False)), kw.get("gradPcmf", 0.0),
        int(kw.get("buoyancy", False)), int(kw.get("boussinesq", False)), kw.get("beta", 0.0),
        kw.get("densit", 1.0), kw.get("tref", 0.0), *g)


def _oracle(m, csr, kw, f, a):
    keys = ("t", "uo", "vo", "wo", "uoo", "voo", "woo")
    return oracle.calcuvw(oracle_mesh(m), csr, _oracle_params(kw), a, f["u"], f["v"], f["w"],
                          f["p"], f["vis"], f["den"], f["dUdxi"], f["dVdxi"], f["dWdxi"],
                          f["dPdxi"], f["flmass"], f["fmi"], f["fmo"], **{k: f[k] for k in keys})


# ---------------------------------------------------------------------------------------
# numpy statement of the reference loops
# ---------------------------------------------------------------------------------------
def _face_value(m, scheme, limiter, f, s, xf, lam, fi, g):
    xc = np.stack([m.xc, m.yc, m.zc], 1)
    if scheme == "cds":
        fxn, fxp = lam, 1.0 - lam
        return fi[f] * fxp + fi[s] * fxn
    if scheme == "cds_corrected":
        fxn, fxp = lam, 1.0 - lam
        xi = [xc[f, k] * fxp + xc[s, k] * fxn for k in range(3)]
        d = [g[f, k] * fxp + g[s, k] * fxn for k in range(3)]
        return fi[f] * fxp + fi[s] * fxn + (d[0] * (xf[0] - xi[0]) + d[1] * (xf[1] - xi[1]) +
                                            d[2] * (xf[2] - xi[2]))
    rf = [xf[k] - xc[f, k] for k in range(3)]
    rs = [xf[k] - xc[s, k] for k in range(3)]
    if scheme == "central":
        r = (g[f, 0] * rf[0] + g[f, 1] * rf[1] + g[f, 2] * rf[2] + g[s, 0] * rs[0] +
             g[s, 1] * rs[1] + g[s, 2] * rs[2])
        return 0.5 * (fi[f] + fi[s] + r)
    if scheme == "second_upwind":
        return fi[f] + (g[f, 0] * rf[0] + g[f, 1] * rf[1] + g[f, 2] * rf[2])
    if scheme == "flux_limiter":
        fxp = 1.0 - lam
        d = [xc[s, k] - xc[f, k] for k in range(3)]
        r = (2 * g[f, 0] * d[0] + 2 * g[f, 1] * d[1] + 2 * g[f, 2] * d[2]) / (fi[s] - fi[f]) - 1.0
        mn, mx = np.minimum, np.maximum
        psi = {
            "smart": lambda: mx(0.0, mn(mn(2.0 * r, 0.75 * r + 0.25), 4.0)),
            "avl": lambda: mx(0.0, mn(mn(1.5 * r, 0.75 * r + 0.25), 2.5)),
            "muscl": lambda: mx(0.0, mn(mn(2.0 * r, 0.5 * r + 0.5), 2.0)),
            "umist": lambda: mx(0.0, mn(mn(mn(2.0 * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.0)),
            "koren": lambda: mx(0.0, mn(mn(2.0 * r, 2.0 / 3.0 * r + 1.0 / 3.0), 2.0)),
            "charm": lambda: (r + np.abs(r)) * (3 * r + 1.0) / (2 * ((r + 1.0) * (r + 1.0))),
            "ospre": lambda: 1.5 * r * (r + 1.0) / (r * r + r + 1.0),
            "uds": lambda: np.ones_like(r),
        }[limiter]()
        return fi[f] + fxp * psi * (fi[s] - fi[f])
    g2 = g[f, 0] * rf[0] + g[f, 1] * rf[1] + g[f, 2] * rf[2]
    gc = (g[f, 0] * rf[0] + g[f, 1] * rf[1] + g[f, 2] * rf[2] + g[s, 0] * rs[0] +
          g[s, 1] * rs[1] + g[s, 2] * rs[2])
    return 0.125 * (0.5 * (fi[f] + fi[s] + gc)) + (1.0 - 0.125) * (fi[f] + g2)


def _calcuvw_numpy(m, csr, kw, f, a_in):
    n, nin = m.numCells, m.numInnerFaces
    P, N = m.owner[:nin] - 1, m.neighbour - 1
    idx = np.empty(2 * nin, np.int64)
    idx[0::2], idx[1::2] = P, N

    def scatter(acc, vals_p, vals_n):
        v = np.empty(2 * nin)
        v[0::2], v[1::2] = vals_p, vals_n
        np.add.at(acc, idx, v)

    scheme, limiter = kw.get("scheme", "muscl"), kw.get("limiter", "uds")
    urf = kw.get("urf", (0.7, 0.7, 0.7))
    urfr, urfm = [1.0 / x for x in urf], [1.0 - x for x in urf]
    cn, bdf = kw.get("cn", False), kw.get("bdf", False)
    dt, bt = kw.get("timestep", 1.0), kw.get("btime", 0.0)
    vol, den = m.vol, f["den"]
    S = [np.zeros(n) for _ in range(3)]
    SP = [np.zeros(n) for _ in range(3)]
    cur = (f["u"], f["v"], f["w"])
    G = (f["dUdxi"], f["dVdxi"], f["dWdxi"])
    # calcPressDiv
    fxn = m.facint
    fxp = 1.0 - fxn
    xc = np.stack([m.xc, m.yc, m.zc])
    xf = np.stack([m.xf[:nin], m.yf[:nin], m.zf[:nin]])
    S3 = np.stack([m.arx[:nin], m.ary[:nin], m.arz[:nin]])
    flat = f["dPdxi"].reshape(-1)
    xi = [xc[k][P] * fxp + xc[k][N] * fxn for k in range(3)]
    df = [flat[P + 3 * k] * fxp + flat[N + 3 * k] * fxn for k in range(3)]
    fie = (f["p"][P] * fxp + f["p"][N] * fxn + df[0] * (xf[0] - xi[0]) + df[1] * (xf[1] - xi[1]) +
           df[2] * (xf[2] - xi[2]))
    for k in range(3):
        scatter(S[k], -(fie * S3[k]), fie * S3[k])
    types = [("ninl", "iInletFacesStart", 0), ("nout", "iOutletFacesStart", 1),
             ("nsym", "iSymmetryFacesStart", 2), ("nwal", "iWallFacesStart", 3),
             ("npru", "iPressOutletFacesStart", 4)]
    bstart, off = {}, n
    for cnt, _, ty in types:
        bstart[ty] = off
        off += m.counts.get(cnt, 0)
    Sb = [m.arx, m.ary, m.arz]
    for cnt, st, ty in types:
        c = m.counts.get(cnt, 0)
        if not c:
            continue
        fc = m.starts[st] + np.arange(c)
        own = m.owner[fc] - 1
        pb = f["p"][bstart[ty] + np.arange(c)]
        for k in range(3):
            np.subtract.at(S[k], own, pb * Sb[k][fc])
    # volume sources
    if kw.get("const_mflux"):
        S[0] = S[0] + kw["gradPcmf"] * vol
    if kw.get("buoyancy"):
        heat = (kw["beta"] * kw["densit"] * (f["t"] - kw["tref"]) * vol if kw.get("boussinesq")
                else (kw["densit"] - den) * vol)
        for k in range(3):
            S[k] = S[k] - kw["grav"][k] * heat
    if bdf:
        apotime = den * vol / dt
        for k, (o, oo) in enumerate((("uo", "uoo"), ("vo", "voo"), ("wo", "woo"))):
            st = apotime * ((1 + bt) * f[o])
            if bt > F32_099:
                st = st - apotime * (0.5 * bt * f[oo])
            S[k] = S[k] + st
            SP[k] = SP[k] + apotime * (1 + 0.5 * bt)
    # facefluxuvw on inner faces
    fm = f["flmass"]
    d = [xc[k][N] - xc[k][P] for k in range(3)]
    dpn = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    are = np.sqrt(S3[0] * S3[0] + S3[1] * S3[1] + S3[2] * S3[2])
    game = f["vis"][P] * fxp + f["vis"][N] * fxn
    de = game * are / dpn
    can = -de + np.minimum(fm, 0.0)
    cap = -de - np.maximum(fm, 0.0)
    vole = d[0] * S3[0] + d[1] * S3[1] + d[2] * S3[2]
    gi, gii = [], []
    for comp in range(3):
        g, fi = G[comp], cur[comp]
        a_ = [g[P, k] * fxp + g[N, k] * fxn for k in range(3)]
        corr = fi[N] - fi[P] - a_[0] * d[0] - a_[1] * d[1] - a_[2] * d[2]
        gi.append(a_)
        gii.append([a_[k] * 1.0 + S3[k] / vole * corr for k in range(3)])
    (uxi, uyi, uzi), (vxi, vyi, vzi), (wxi, wyi, wzi) = gii
    ax, ay, az = S3
    fde = [game * ((uxi + uxi) * ax + (uyi + vxi) * ay + (uzi + wxi) * az),
           game * ((uyi + vxi) * ax + (vyi + vyi) * ay + (vzi + wyi) * az),
           game * ((uzi + wxi) * ax + (wyi + vzi) * ay + (wzi + wzi) * az)]
    fdi = [game * are / dpn * (gi[c][0] * d[0] + gi[c][1] * d[1] + gi[c][2] * d[2])
           for c in range(3)]
    pos = fm >= 0.0
    first, second = np.where(pos, P, N), np.where(pos, N, P)
    lam = np.where(pos, fxp, fxn)
    gds = kw.get("gds", 1.0)
    for comp in range(3):
        fi = cur[comp]
        uds = np.maximum(fm, 0.0) * fi[P] + np.minimum(fm, 0.0) * fi[N]
        fv = _face_value(m, scheme, limiter, first, second, xf, lam, fi, G[comp])
        src = -gds * (fm * fv - uds) + fde[comp] - fdi[comp]
        scatter(S[comp], src, -src)
    a = a_in.copy()
    a[csr.slot_pn - 1] = can
    a[csr.slot_np - 1] = cap
    # inlet / outlet
    for cnt, st, ty, fl in (("ninl", "iInletFacesStart", 0, f["fmi"]),
                            ("nout", "iOutletFacesStart", 1, f["fmo"])):
        c = m.counts.get(cnt, 0)
        if not c:
            continue
        fc = m.starts[st] + np.arange(c)
        own = m.owner[fc] - 1
        b = bstart[ty] + np.arange(c)
        r = [np.array([m.xf, m.yf, m.zf][k][fc]) - xc[k][own] for k in range(3)]
        dp = np.sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])
        ar = np.sqrt(m.arx[fc] * m.arx[fc] + m.ary[fc] * m.ary[fc] + m.arz[fc] * m.arz[fc])
        cb = -(f["vis"][b] * ar / dp) + np.minimum(fl, 0.0)
        for k in range(3):
            np.subtract.at(SP[k], own, cb)
            np.subtract.at(S[k], own, cb * cur[k][b])
    # symmetry, wall
    for cnt, st, ty in (("nsym", "iSymmetryFacesStart", 2), ("nwal", "iWallFacesStart", 3)):
        c = m.counts.get(cnt, 0)
        if not c:
            continue
        fc = m.starts[st] + np.arange(c)
        own = m.owner[fc] - 1
        b = bstart[ty] + np.arange(c)
        A = [m.arx[fc], m.ary[fc], m.arz[fc]]
        ar = np.sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2])
        nv = [A[k] / ar for k in range(3)]
        fxyz = [m.xf[fc], m.yf[fc], m.zf[fc]]
        dn = ((fxyz[0] - xc[0][own]) * nv[0] + (fxyz[1] - xc[1][own]) * nv[1] +
              (fxyz[2] - xc[2][own]) * nv[2])
        srd = ar / dn
        dd = [xc[k][own] - fxyz[k] for k in range(3)]
        dpb = np.sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2])
        pb = [cur[k][own] - cur[k][b] for k in range(3)]
        visc = f["vis"][b] if ty == 2 else np.full(c, kw.get("viscos", 1e-3))
        cf = visc * srd
        vsol = visc * ar / dpb
        if ty == 2:
            fdne = 2 * cf * (pb[0] * nv[0] + pb[1] * nv[1] + pb[2] * nv[2])
        else:
            vnp = pb[0] * nv[0] + pb[1] * nv[1] + pb[2] * nv[2]
        for k in range(3):
            np.add.at(SP[k], own, vsol)
            # su = su + vsol*u - x: add the two terms one after the other
            for i in range(c):
                S[k][own[i]] = S[k][own[i]] + vsol[i] * cur[k][own[i]] - (
                    fdne[i] * nv[k][i] if ty == 2 else cf[i] * (pb[k][i] - vnp[i] * nv[k][i]))
    if cn:
        a = 0.5 * a
    rows = [slice(csr.ioffset[i] - 1, csr.ioffset[i + 1] - 1) for i in range(n)]
    dg = csr.diag - 1

    def row_sums():
        return np.array([sum(a[r], 0.0) for r in rows])

    old = (f["uo"], f["vo"], f["wo"])
    other = np.empty(2 * nin, np.int64)
    other[0::2], other[1::2] = N, P
    slots = np.empty(2 * nin, np.int64)
    slots[0::2], slots[1::2] = csr.slot_pn - 1, csr.slot_np - 1
    rhs, ap, dvw = np.zeros((3, n)), np.zeros((3, n)), np.zeros((2, n))
    su = S[0]
    du = None
    for comp in range(3):
        if cn:
            np.subtract.at(S[comp], idx, a[slots] * old[comp][other])
            apotime = den * vol / dt
            S[comp] = S[comp] + (apotime + (row_sums() - a[dg])) * old[comp]
            SP[comp] = SP[comp] + apotime
            if comp == 0:
                su = S[0]
        if comp > 0:
            a[dg] = 0.0
        diag = (SP[comp] - (row_sums() - a[dg])) * urfr[comp]
        a[dg] = diag
        rhs[comp] = (su if comp == 0 else S[comp]) + urfm[comp] * diag * cur[comp][:n]
        ap[comp] = 1.0 / (diag + SMALL)
        if comp == 0:
            du = diag.copy()
        else:
            dvw[comp - 1] = diag
    a[dg] = du
    return a, dvw, rhs, ap


@pytest.mark.parametrize("k", [0, 4, 5, 9, 13, 14, 15, 16])
def test_oracle_calcuvw_restates_the_loops(k):
    kw = OPTS[k]
    from tests.meshes import mixed_patch_mesh

    for m in (hex_mesh(5, 0.2), fixture_mesh("pitzdaily"), mixed_patch_mesh(6)):
        csr = oracle_csr(m)
        f, a = _fields(m, 3), _a_in(m, 3)
        got = _oracle(m, csr, kw, f, a)
        ref = _calcuvw_numpy(m, csr, kw, f, a)
        for x, y, name in zip(got, ref, ("a", "diag_vw", "rhs", "ap")):
            assert np.array_equal(x, y), (kw, name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pitzdaily", "hex8", "hexmix8"])
def test_calcuvw_bit_exact(name):
    from tests.meshes import mesh_by_name

    m = mesh_by_name(name)
    c = fcg.Context(m)
    csr = oracle_csr(m)
    f, a = _fields(m, 5), _a_in(m, 5)
    keys = ("u", "v", "w", "p", "vis", "den", "dUdxi", "dVdxi", "dWdxi", "dPdxi", "flmass")
    for kw in OPTS:
        got = c.calcuvw(*[f[k] for k in keys], a, f["fmi"], f["fmo"], t=f["t"], uo=f["uo"],
                        vo=f["vo"], wo=f["wo"], uoo=f["uoo"], voo=f["voo"], woo=f["woo"], **kw)
        ref = _oracle(m, csr, kw, f, a)
        for key, r in zip(("a", "diag_vw", "rhs", "ap"), ref):
            assert np.array_equal(got[key], r), (kw, key)
    c.close()


@pytest.mark.gpu
def test_momentum_systems_solve_like_calcuvw():
    """The three solves of calcuvw (:441,498,556) on the assembled systems, GPU BiCGStab
    against the oracle's, and the same three systems in one multi-RHS call."""
    m = fixture_mesh("pitzdaily")
    c = fcg.Context(m)
    csr = oracle_csr(m)
    f, a = _fields(m, 7), _a_in(m, 7)
    keys = ("u", "v", "w", "p", "vis", "den", "dUdxi", "dVdxi", "dWdxi", "dPdxi", "flmass")
    asm = c.calcuvw(*[f[k] for k in keys], a, f["fmi"], f["fmo"], bdf=True, timestep=0.01,
                    uo=f["uo"], vo=f["vo"], wo=f["wo"])
    a3, rhs = c.uvw_systems(asm)
    n = m.numCells
    sols = []
    for k, x0 in enumerate((f["u"], f["v"], f["w"])):
        g = c.bicgstab(a3[k], rhs[k], x0[:n], 1e-8, 500)
        o = oracle.bicgstab(csr, a3[k], rhs[k], x0[:n].copy(), 1e-8, 500)
        assert g.converged and abs(g.iters - o.iters) <= 1
        rel = np.abs(g.fi - o.fi).max() / np.abs(o.fi).max()
        assert rel < 1e-8, k
        sols.append(g.fi)
    fi, reps = c.bicgstab_multi(a3, rhs, np.stack([x[:n] for x in (f["u"], f["v"], f["w"])]),
                                1e-10, 500)
    for k in range(3):
        assert reps[k].converged and reps[k].l2_rel < 1e-9
        assert np.abs(fi[k] - sols[k]).max() / np.abs(sols[k]).max() < 1e-6
    c.close()
