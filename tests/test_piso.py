"""The PISO pressure path (PISO_multiple_correction.f90:83-307).

Its own steps are get_rAU_x_UEqnH, the facefluxmass_piso assembly, adjustMassFlow, the
reference-pressure row and the PISO velocity correction. The CPU tests pin the oracle's
restatement against a direct numpy statement of the reference loops. The GPU tests
compare every step with the oracle bit for bit, and one corrector chained as the
reference chains it.

The numpy statements use np.subtract.at over the interleaved (owner, neighbour) index
list of the face loop. ufunc.at applies the updates one after another in index order,
so each cell receives its terms in the reference's face order."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import oracle
from tests.meshes import fixture_mesh, hex_mesh, oracle_csr, oracle_mesh, seeded_fields

F32_099 = float(np.float32(0.99))  # a default-real literal in get_rAU_x_UEqnH.f90:73

FLAGS = [
    dict(),
    dict(bdf=True, btime=0.0, timestep=0.01),
    dict(bdf=True, btime=1.0, timestep=0.02, cn=True),
    dict(cn=True, timestep=0.05),
    dict(buoyancy=True, boussinesq=True, beta=3e-3, densit=1.2, tref=290.0,
         grav=(0.0, -9.81, 0.5)),
    dict(buoyancy=True, boussinesq=False, densit=1.1, grav=(0.3, -9.81, 0.0), bdf=True,
         btime=0.0, timestep=0.1),
]


def _params(kw):
    g = kw.get("grav", (0.0, 0.0, 0.0))
    return oracle.HbyaParams(kw.get("timestep", 1.0), kw.get("btime", 0.0),
                             int(kw.get("bdf", False)), int(kw.get("cn", False)),
                             int(kw.get("buoyancy", False)), int(kw.get("boussinesq", False)),
                             kw.get("beta", 0.0), kw.get("densit", 1.0), kw.get("tref", 0.0), *g)


def _momentum(m, csr, seed):
    """A momentum-like matrix on the mesh's pattern: negative off-diagonals, a dominant
    diagonal, values U-distributed."""
    rng = np.random.default_rng(seed)
    h = -rng.uniform(0.5, 1.5, csr.nnz)
    rows = np.repeat(np.arange(m.numCells), np.diff(csr.ioffset))
    off = np.zeros(m.numCells)
    mask = np.ones(csr.nnz, bool)
    mask[csr.diag - 1] = False
    np.add.at(off, rows[mask], -h[mask])
    h[csr.diag - 1] = off * 1.05 + 0.1
    return h


def _old_fields(m, seed):
    n = m.numCells
    return dict(t=280.0 + 20.0 * fcg.uniform(seed, 40, n),
                uo=fcg.uniform(seed, 41, n), vo=fcg.uniform(seed, 42, n),
                wo=fcg.uniform(seed, 43, n), uoo=fcg.uniform(seed, 44, n),
                voo=fcg.uniform(seed, 45, n), woo=fcg.uniform(seed, 46, n))


def _hbya_numpy(m, csr, kw, h, f, old):
    """get_rAU_x_UEqnH.f90:32-206 in numpy."""
    n, nin = m.numCells, m.numInnerFaces
    vol, den = m.vol, f["den"][:n]
    s = [np.zeros(n) for _ in range(3)]
    if kw.get("buoyancy"):
        if kw.get("boussinesq"):
            heat = kw["beta"] * kw["densit"] * (old["t"] - kw["tref"]) * vol
        else:
            heat = (kw["densit"] - den) * vol
        s = [s[k] - kw["grav"][k] * heat for k in range(3)]
    if kw.get("bdf"):
        apotime = den * vol / kw["timestep"]
        bt = kw["btime"]
        for k, (o, oo) in enumerate((("uo", "uoo"), ("vo", "voo"), ("wo", "woo"))):
            st = apotime * ((1 + bt) * old[o])
            if bt > F32_099:
                st = st - apotime * (0.5 * bt * old[oo])
            s[k] = s[k] + st
    P, N = m.owner[:nin] - 1, m.neighbour - 1
    idx = np.empty(2 * nin, np.int64)
    idx[0::2], idx[1::2] = P, N
    hk = np.empty(2 * nin)
    hk[0::2], hk[1::2] = h[csr.slot_pn - 1], h[csr.slot_np - 1]
    other = np.empty(2 * nin, np.int64)
    other[0::2], other[1::2] = N, P
    cur = (f["u"], f["v"], f["w"])
    for k, o in enumerate(("uo", "vo", "wo")):
        if kw.get("cn"):
            np.subtract.at(s[k], idx, hk * old[o][other])
            apotime = den * vol / kw["timestep"]
            offd = np.array([sum(h[csr.ioffset[i] - 1:csr.ioffset[i + 1] - 1], 0.0)
                             for i in range(n)]) - h[csr.diag - 1]
            s[k] = s[k] + (apotime + offd) * old[o]
        np.subtract.at(s[k], idx, hk * cur[k][other])
    ap = (f["apu"], f["apv"], f["apw"])
    return [ap[k] * s[k] for k in range(3)] + s


@pytest.mark.parametrize("k", range(len(FLAGS)))
def test_oracle_hbya_restates_the_loops(k):
    m = hex_mesh(5, 0.2)
    om, csr = oracle_mesh(m), oracle_csr(m)
    f, old, kw = seeded_fields(m, seed=4), _old_fields(m, 4), FLAGS[k]
    h = _momentum(m, csr, 1)
    got = oracle.piso_hbya(om, csr, _params(kw), h, f["den"], f["apu"], f["apv"], f["apw"],
                           f["u"], f["v"], f["w"], **old)
    ref = _hbya_numpy(m, csr, kw, h, f, old)
    n = m.numCells
    for x, y in zip(got[:3], ref[:3]):
        assert np.array_equal(x[:n], y)
    for x, y in zip(got[3:], ref[3:]):
        assert np.array_equal(x, y)
    # the boundary slots of u, v, w are left alone
    assert np.array_equal(got[0][n:], f["u"][n:])


def test_oracle_piso_assembly_and_mass_flow_restate_the_loops():
    m = fixture_mesh("pitzdaily")
    om, csr = oracle_mesh(m), oracle_csr(m)
    f = seeded_fields(m, seed=6)
    n, nin = m.numCells, m.numInnerFaces
    a, su, flm = oracle.facefluxmass_piso(om, csr, f["u"], f["v"], f["w"], f["dUdxi"],
                                          f["dVdxi"], f["dWdxi"], f["apu"], f["den"])
    P, N = m.owner[:nin] - 1, m.neighbour - 1
    fxn = m.facint
    fxp = 1.0 - fxn
    d = np.stack([m.xc[N] - m.xc[P], m.yc[N] - m.yc[P], m.zc[N] - m.zc[P]])
    S = np.stack([m.arx[:nin], m.ary[:nin], m.arz[:nin]])
    dpn = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    are = np.sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2])
    dene = f["den"][P] * fxp + f["den"][N] * fxn
    cap = -(dene * (fxp * m.vol[P] * f["apu"][P] + fxn * m.vol[N] * f["apu"][N]) * are / dpn)
    xf = np.stack([m.xf[:nin], m.yf[:nin], m.zf[:nin]])
    xc = np.stack([m.xc, m.yc, m.zc])

    def central(phi, g):  # interpolation.f90:145-199
        r = (g[P, 0] * (xf[0] - xc[0][P]) + g[P, 1] * (xf[1] - xc[1][P]) +
             g[P, 2] * (xf[2] - xc[2][P]) + g[N, 0] * (xf[0] - xc[0][N]) +
             g[N, 1] * (xf[1] - xc[1][N]) + g[N, 2] * (xf[2] - xc[2][N]))
        return 0.5 * (phi[P] + phi[N] + r)

    ui, vi, wi = (central(f[c], f[g]) for c, g in (("u", "dUdxi"), ("v", "dVdxi"),
                                                  ("w", "dWdxi")))
    fm = dene * (ui * S[0] + vi * S[1] + wi * S[2])
    assert np.array_equal(flm, fm)
    assert np.array_equal(a[csr.slot_pn - 1], cap) and np.array_equal(a[csr.slot_np - 1], cap)
    dg, s = np.zeros(n), np.zeros(n)
    idx = np.empty(2 * nin, np.int64)
    idx[0::2], idx[1::2] = P, N
    vals = np.repeat(cap, 2)
    np.subtract.at(dg, idx, vals)
    sv = np.empty(2 * nin)
    sv[0::2], sv[1::2] = -fm, fm
    np.add.at(s, idx, sv)
    assert np.array_equal(a[csr.diag - 1], dg) and np.array_equal(su, s)

    # adjustMassFlow.f90 (pitzDaily has an inlet and an outlet)
    ninl, nout = m.counts["ninl"], m.counts["nout"]
    assert ninl > 0 and nout > 0
    fmi = fcg.uniform(5, 7, ninl, 0.0, 1.0)
    u2, v2, w2, fmo, su2 = oracle.adjust_mass_flow(om, f["den"], 0.9, fmi, f["u"], f["v"],
                                                   f["w"], su)
    ref_su, uu = su.copy(), f["u"].copy()
    ist, ost = m.starts["iInletFacesStart"], m.starts["iOutletFacesStart"]
    for i in range(ninl):
        ref_su[m.owner[ist + i] - 1] -= fmi[i]
    flowo, fmo_ref = 0.0, np.zeros(nout)
    bo = n + ninl
    for i in range(nout):
        fc = ost + i
        c = m.owner[fc] - 1
        uu[bo + i] = f["u"][c]
        fmo_ref[i] = f["den"][c] * (f["u"][c] * m.arx[fc] + f["v"][c] * m.ary[fc] +
                                    f["w"][c] * m.arz[fc])
        flowo = flowo + fmo_ref[i]
    fac = 0.9 / (flowo + float(np.float32(1e-20)))
    for i in range(nout):
        fmo_ref[i] *= fac
        uu[bo + i] *= fac
        ref_su[m.owner[ost + i] - 1] -= fmo_ref[i]
    assert np.array_equal(fmo, fmo_ref) and np.array_equal(su2, ref_su)
    assert np.array_equal(u2, uu)

    # PISO :188-192 and :300-304
    a3, su3 = oracle.set_reference_pressure(csr, 7, f["p"], a, su)
    row = slice(csr.ioffset[6] - 1, csr.ioffset[7] - 1)
    assert np.all(a3[row][np.arange(row.start, row.stop) != csr.diag[6] - 1] == 0)
    assert a3[csr.diag[6] - 1] == 1.0 and su3[6] == f["p"][6]
    uc, vc, wc = oracle.correct_velocity_piso(om, f["dPdxi"], f["apu"], f["apv"], f["apw"],
                                              f["u"], f["v"], f["w"])
    assert np.array_equal(uc[:n], f["u"][:n] - f["apu"] * f["dPdxi"][:, 0] * m.vol)
    assert np.array_equal(wc[:n], f["w"][:n] - f["apw"] * f["dPdxi"][:, 2] * m.vol)


MESHES = ["pitzdaily", "hex8", "hexmix8"]


def _mesh(name):
    from tests.meshes import mesh_by_name

    return mesh_by_name(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_piso_hbya_bit_exact(name):
    m = _mesh(name)
    c = fcg.Context(m)
    om, csr = oracle_mesh(m), oracle_csr(m)
    f, old = seeded_fields(m, seed=8), _old_fields(m, 8)
    h = _momentum(m, csr, 2)
    for kw in FLAGS:
        got = c.piso_hbya(h, f["u"], f["v"], f["w"], f["apu"], f["apv"], f["apw"], f["den"],
                          **kw, **old)
        ref = oracle.piso_hbya(om, csr, _params(kw), h, f["den"], f["apu"], f["apv"], f["apw"],
                               f["u"], f["v"], f["w"], **old)
        for x, y in zip(got, ref):
            assert np.array_equal(x, y), kw
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_piso_assembly_mass_flow_reference_and_velocity_bit_exact(name):
    m = _mesh(name)
    c = fcg.Context(m)
    om, csr = oracle_mesh(m), oracle_csr(m)
    f = seeded_fields(m, seed=9)
    got = c.facefluxmass_piso(f["u"], f["v"], f["w"], f["dUdxi"], f["dVdxi"], f["dWdxi"],
                              f["apu"], f["den"])
    ref = oracle.facefluxmass_piso(om, csr, f["u"], f["v"], f["w"], f["dUdxi"], f["dVdxi"],
                                   f["dWdxi"], f["apu"], f["den"])
    for x, y in zip(got, ref):
        assert np.array_equal(x, y)
    a, su = ref[0], ref[1]
    fmi = fcg.uniform(9, 3, m.counts.get("ninl", 0), 0.0, 1.0)
    g = c.adjust_mass_flow(f["den"], 0.8, fmi, f["u"], f["v"], f["w"], su)
    r = oracle.adjust_mass_flow(om, f["den"], 0.8, fmi, f["u"], f["v"], f["w"], su)
    for x, y in zip(g, r):
        assert np.array_equal(x, y)
    for ref_cell in (1, m.numCells // 2, m.numCells):
        ga, gs = c.set_reference_pressure(ref_cell, f["p"], a, su)
        ra, rs = oracle.set_reference_pressure(csr, ref_cell, f["p"], a, su)
        assert np.array_equal(ga, ra) and np.array_equal(gs, rs)
    g = c.correct_velocity_piso(f["dPdxi"], f["apu"], f["apv"], f["apw"], f["u"], f["v"],
                                f["w"])
    r = oracle.correct_velocity_piso(om, f["dPdxi"], f["apu"], f["apv"], f["apw"], f["u"],
                                     f["v"], f["w"])
    for x, y in zip(g, r):
        assert np.array_equal(x, y)
    c.close()


NIPGRAD = 2


def piso_corrector(ops, m, csr, f, h, ncorr, npcor, flomas, fmi, pref=1, sor=1e-8, nsw=2000):
    """PISO_multiple_correction.f90:87-310 through `ops` (the library or the oracle)."""
    n = m.numCells
    u, v, w, p = f["u"].copy(), f["v"].copy(), f["w"].copy(), f["p"].copy()
    pp = p.copy()
    iters, errs = [], []
    for _ in range(ncorr):
        u, v, w = ops.hbya(h, u, v, w)
        dU, dV, dW = ops.grad(u), ops.grad(v), ops.grad(w)
        a, su, flmass = ops.assemble(u, v, w, dU, dV, dW)
        u, v, w, fmo, su = ops.adjust(flomas, fmi, u, v, w, su)
        a, su = ops.pref(pref, p, a, su)
        for ipcorr in range(1, npcor + 1):
            fi, it = ops.iccg(a, su, pp[:n], sor, nsw)
            iters.append(it)
            pp = np.concatenate([fi, pp[n:]])
            if ipcorr == npcor:
                flmass = ops.flux_correct(a, pp, flmass)
            errs.append(ops.continuity(flmass, fmi, fmo))
        p = pp.copy()
        for istage in range(1, NIPGRAD + 1):
            p = ops.bpres(p, f["dPdxi"] if istage == 1 else dP, istage)
            dP = ops.grad(p)
        u, v, w = ops.correct_velocity(dP, u, v, w)
        u, v, w, fmo = ops.correct_bc(flomas, u, v, w)
    return dict(u=u, v=v, w=w, p=p, flmass=flmass, dP=dP, iters=iters, errs=errs)


class _GpuOps:
    def __init__(self, c, f):
        self.c, self.f = c, f

    def hbya(self, h, u, v, w):
        f = self.f
        return self.c.piso_hbya(h, u, v, w, f["apu"], f["apv"], f["apw"], f["den"])[:3]

    def grad(self, phi):
        return self.c.grad(phi, "gauss")

    def assemble(self, u, v, w, dU, dV, dW):
        return self.c.facefluxmass_piso(u, v, w, dU, dV, dW, self.f["apu"], self.f["den"])

    def adjust(self, flomas, fmi, u, v, w, su):
        return self.c.adjust_mass_flow(self.f["den"], flomas, fmi, u, v, w, su)

    def pref(self, ref, p, a, su):
        return self.c.set_reference_pressure(ref, p, a, su)

    def iccg(self, a, su, x0, sor, nsw):
        r = self.c.iccg(a, su, x0, sor, nsw)
        return r.fi, r.iters

    def flux_correct(self, a, pp, flmass):
        return self.c.flux_correct(a, pp, flmass)

    def continuity(self, flmass, fmi, fmo):
        return self.c.continuity_errors(flmass, fmi, fmo)[1:]

    def bpres(self, p, dP, istage):
        return self.c.bpres(p, dP, istage)

    def correct_velocity(self, dP, u, v, w):
        f = self.f
        return self.c.correct_velocity_piso(dP, f["apu"], f["apv"], f["apw"], u, v, w)

    def correct_bc(self, flomas, u, v, w):
        return self.c.correct_bc_velocity(self.f["den"], flomas, u, v, w)


class _OracleOps:
    def __init__(self, m, f):
        self.om, self.csr, self.f = oracle_mesh(m), oracle_csr(m), f

    def hbya(self, h, u, v, w):
        f = self.f
        return oracle.piso_hbya(self.om, self.csr, _params({}), h, f["den"], f["apu"], f["apv"],
                                f["apw"], u, v, w)[:3]

    def grad(self, phi):
        return oracle.grad_gauss(self.om, phi, 1)

    def assemble(self, u, v, w, dU, dV, dW):
        return oracle.facefluxmass_piso(self.om, self.csr, u, v, w, dU, dV, dW, self.f["apu"],
                                        self.f["den"])

    def adjust(self, flomas, fmi, u, v, w, su):
        return oracle.adjust_mass_flow(self.om, self.f["den"], flomas, fmi, u, v, w, su)

    def pref(self, ref, p, a, su):
        return oracle.set_reference_pressure(self.csr, ref, p, a, su)

    def iccg(self, a, su, x0, sor, nsw):
        r = oracle.iccg(self.csr, a, su, x0, sor, nsw)
        return r.fi, r.iters

    def flux_correct(self, a, pp, flmass):
        return oracle.flux_correct(self.om, self.csr, a, pp, flmass)

    def continuity(self, flmass, fmi, fmo):
        return oracle.continuity_errors(self.om, flmass, fmi, fmo)[1:]

    def bpres(self, p, dP, istage):
        return oracle.bpres(self.om, p, dP, istage)

    def correct_velocity(self, dP, u, v, w):
        f = self.f
        return oracle.correct_velocity_piso(self.om, dP, f["apu"], f["apv"], f["apw"], u, v, w)

    def correct_bc(self, flomas, u, v, w):
        return oracle.correct_bc_velocity(self.om, self.f["den"], flomas, u, v, w)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
def test_piso_corrector_matches_oracle():
    """Two PISO correctors with two pressure corrections each on the pitzDaily mesh
    (inlet, outlet, walls; the pressure level fixed by pRefCell)."""
    m = fixture_mesh("pitzdaily")
    c = fcg.Context(m)
    f = seeded_fields(m, seed=12)
    csr = oracle_csr(m)
    h = _momentum(m, csr, 3)
    fmi = fcg.uniform(12, 5, m.counts["ninl"], 0.0, 1.0) * 1e-3
    flomas = float(fmi.sum())
    g = piso_corrector(_GpuOps(c, f), m, csr, f, h, 2, 2, flomas, fmi)
    o = piso_corrector(_OracleOps(m, f), m, csr, f, h, 2, 2, flomas, fmi)
    assert all(abs(i - j) <= 1 for i, j in zip(g["iters"], o["iters"]))
    for k in ("u", "v", "w", "p", "flmass", "dP"):
        assert _rel(g[k], o[k]) < 1e-8, k
    for (gl, gg), (ol, og) in zip(g["errs"], o["errs"]):
        assert gl == pytest.approx(ol, rel=1e-8, abs=1e-14)
    c.close()
