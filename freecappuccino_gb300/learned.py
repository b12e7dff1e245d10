"""Learned preconditioner for the pressure solve and the flexible CG that uses it.

No reference counterpart: the reference solves the pressure equation with dpcg/iccg
(dpcg.f90, iccg.f90).  Here a small message-passing network (libfcgpu.so, learned.cu)
approximates the inverse of the Jacobi-scaled pressure matrix and serves as the
preconditioner of a flexible CG; plain FP64 DPCG stays the fallback (taken when the
FCG stalls) and the check on the result (the stop test is dpcg.f90's L1 test on the
FP64 residual).  Training data are (residual, error) pairs of DPCG iterates on seeded
jittered meshes with a smoothed log-uniform diffusivity; training runs on the GPU
through the library's own forward, backward and Adam kernels.

Vectors of the network live in the scaled system: r = D^-1/2 (su - A x) and
e = D^1/2 (x* - x), FP32, D = diag(A).
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .mesh import Mesh, hex_mesh, uniform
from .pressure import Context, SolveResult, _host, _is_torch, _ptr

WIDTH, LAYERS, FEATURES, PARAMS = 32, 6, 6, 12737
# default checkpoint shipped with the package (trained by train_default())
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                               "lp_c32_l6.fcglp")


def _f32(x):
    if _is_torch(x):
        import torch

        return x.to(torch.float32).contiguous()
    return np.ascontiguousarray(x, dtype=np.float32)


def _like(x):
    if _is_torch(x):
        import torch

        return torch.empty_like(x)
    return np.zeros_like(x)


class LearnedPreconditioner:
    """An fcg_learned handle: FP32 weights and Adam state on one device."""

    def __init__(self, device: int = 0, seed: int = 0, path: str | None = None):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.fcg_lp_create(int(device), int(seed), C.byref(h))
        if rc != 0:
            raise _lib.FcgError(rc, "fcg_lp_create", "no usable sm_103a CUDA device")
        self.h = h
        if path is not None:
            self.load(path)

    def _check(self, rc, where):
        if rc != 0:
            raise _lib.FcgError(rc, where, self.lib.fcg_lp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fcg_lp_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    # -- weights ------------------------------------------------------------------
    @property
    def weights(self) -> np.ndarray:
        w = np.zeros(PARAMS, np.float32)
        self._check(self.lib.fcg_lp_get_weights(self.h, _ptr(w), PARAMS), "fcg_lp_get_weights")
        return w

    @weights.setter
    def weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.fcg_lp_set_weights(self.h, _ptr(w), int(w.size)), "fcg_lp_set_weights")

    def save(self, path: str):
        self._check(self.lib.fcg_lp_save(self.h, os.fsencode(path)), "fcg_lp_save")

    def load(self, path: str):
        self._check(self.lib.fcg_lp_load(self.h, os.fsencode(path)), "fcg_lp_load")

    # -- network ------------------------------------------------------------------
    def set_matrix(self, ctx: Context, a):
        ctx._follow(a)
        self._check(self.lib.fcg_lp_set_matrix(self.h, ctx.h, _ptr(_host(a))), "fcg_lp_set_matrix")

    def features(self, ctx: Context) -> np.ndarray:
        """Per-cell inputs of the network as (numCells, FEATURES)."""
        out = np.zeros((FEATURES, ctx.n), np.float32)
        self._check(self.lib.fcg_lp_features(self.h, ctx.h, _ptr(out)), "fcg_lp_features")
        return np.ascontiguousarray(out.T)

    def apply(self, ctx: Context, r):
        r = _f32(r)
        ctx._follow(r)
        if _is_torch(r):
            import torch

            z = torch.empty_like(r)
        else:
            z = np.zeros_like(r)
        self._check(self.lib.fcg_lp_apply(self.h, ctx.h, _ptr(r), _ptr(z)), "fcg_lp_apply")
        return z

    def loss_grad(self, ctx: Context, r, e):
        r, e = _f32(r), _f32(e)
        ctx._follow(r, e)
        loss = C.c_float()
        g = np.zeros(PARAMS, np.float32)
        self._check(self.lib.fcg_lp_loss_grad(self.h, ctx.h, _ptr(r), _ptr(e), C.byref(loss),
                                              _ptr(g)), "fcg_lp_loss_grad")
        return float(loss.value), g

    def train_step(self, ctx: Context, r, e, lr: float) -> float:
        r, e = _f32(r), _f32(e)
        ctx._follow(r, e)
        loss = C.c_float()
        self._check(self.lib.fcg_lp_train_step(self.h, ctx.h, _ptr(r), _ptr(e), float(lr),
                                               C.byref(loss)), "fcg_lp_train_step")
        return float(loss.value)

    def last_solve_stats(self) -> dict:
        """FCG iterations and FP64 residual replacements of the last solve."""
        it, up = C.c_int(), C.c_int()
        self._check(self.lib.fcg_lp_last_solve_stats(self.h, C.byref(it), C.byref(up)),
                    "fcg_lp_last_solve_stats")
        return {"iters": it.value, "updates": up.value}

    def profile(self, ctx: Context, r, reps: int = 10) -> dict:
        """Mean milliseconds of each kernel of one forward pass on r."""
        r = _f32(r)
        ctx._follow(r)
        ms = (C.c_double * 16)()
        nu = C.c_int()
        self._check(self.lib.fcg_lp_profile(self.h, ctx.h, _ptr(r), int(reps), ms, 16,
                                            C.byref(nu)), "fcg_lp_profile")
        names = ["k_lp_rms", "k_lp_embed"] + [f"k_lp_layer#{l + 1}" for l in range(LAYERS)]
        names.append("k_lp_out")
        return {names[i]: ms[i] for i in range(nu.value)}

    def layer_form(self, ctx: Context) -> dict:
        """Which form of the layer kernel inference runs on ctx's mesh: "planes" (the
        cells form a lexicographic hex block; planes staged by TMA copies) or "gather"
        (the sliced gather, any mesh).  Both give the same bits."""
        form = C.c_int()
        dims = (C.c_int * 3)()
        self._check(self.lib.fcg_lp_layer_form(self.h, ctx.h, C.byref(form), dims),
                    "fcg_lp_layer_form")
        return {"form": "planes" if form.value == 1 else "gather", "dims": tuple(dims)}

    def set_loss(self, kind: str = "residual"):
        """Training loss: "residual" (|Ahat N(r) - r|^2 / |r|^2, the default), "energy"
        ((N(r)-e).Ahat(N(r)-e) / e.Ahat e) or "cycle" ((M(r)-e).Ahat(M(r)-e) / e.Ahat e
        with M the network followed by the coarse-grid correction)."""
        k = {"energy": 0, "residual": 1, "cycle": 2}[kind]
        self._check(self.lib.fcg_lp_set_loss(self.h, k), "fcg_lp_set_loss")

    def set_fcg_options(self, directions: int = 8, ru_every: int = 50, stall_window: int = 400,
                        stall_factor: float = 0.5):
        self._check(self.lib.fcg_lp_set_fcg_options(self.h, int(directions), int(ru_every),
                                                    int(stall_window), float(stall_factor)),
                    "fcg_lp_set_fcg_options")

    # -- coarse-grid correction ---------------------------------------------------
    @property
    def multilevel(self) -> dict:
        """Options of the coarse-grid correction (fcg_lp_multilevel) as a dict."""
        o = _lib.Multilevel()
        self._check(self.lib.fcg_lp_get_multilevel(self.h, C.byref(o)), "fcg_lp_get_multilevel")
        d = {k: getattr(o, k) for k, _ in _lib.Multilevel._fields_}
        d["smoother"] = "jacobi" if o.smoother == _lib.SMOOTH_JACOBI else "network"
        return d

    def set_multilevel(self, enabled: bool | None = None, smoother: str | None = None,
                       sweeps: int | None = None, max_levels: int | None = None,
                       dense_max: int | None = None, alpha: float | None = None,
                       omega: float | None = None, smoothed: bool | None = None):
        """Changes the given options of the coarse-grid correction; smoother is "network"
        (the default) or "jacobi" (the same cycle without the network)."""
        cur = self.multilevel
        new = dict(enabled=enabled, smoother=smoother, sweeps=sweeps, max_levels=max_levels,
                   dense_max=dense_max, alpha=alpha, omega=omega, smoothed=smoothed)
        for k, v in new.items():
            if v is not None:
                cur[k] = v
        o = _lib.Multilevel(int(bool(cur["enabled"])),
                            {"network": _lib.SMOOTH_NETWORK, "jacobi": _lib.SMOOTH_JACOBI}[cur["smoother"]],
                            int(cur["sweeps"]), int(cur["max_levels"]), int(cur["dense_max"]),
                            float(cur["alpha"]), float(cur["omega"]), int(bool(cur["smoothed"])))
        self._check(self.lib.fcg_lp_set_multilevel(self.h, C.byref(o)), "fcg_lp_set_multilevel")

    def hierarchy(self, ctx: Context) -> dict:
        """Levels (the fine one first): cells and entries of each, the seconds the
        construction took and where it ran ("device" or "host")."""
        nl = C.c_int()
        cells = (C.c_int * _lib.MAX_LEVELS)()
        ent = (C.c_longlong * _lib.MAX_LEVELS)()
        sec = C.c_double()
        dev = C.c_int()
        self._check(self.lib.fcg_lp_hierarchy_info(self.h, ctx.h, C.byref(nl), cells, ent,
                                                   C.byref(sec)), "fcg_lp_hierarchy_info")
        self._check(self.lib.fcg_lp_hierarchy_built_on(self.h, ctx.h, C.byref(dev)),
                    "fcg_lp_hierarchy_built_on")
        return {"cells": list(cells[:nl.value]), "entries": list(ent[:nl.value]),
                "setup_seconds": sec.value, "built_on": "device" if dev.value else "host"}

    def hierarchy_level(self, ctx: Context, level: int) -> dict:
        """Arrays of coarse level `level` (1-based below the fine one), 0-based."""
        info = self.hierarchy(ctx)
        n_above, n, nnz = info["cells"][level - 1], info["cells"][level], info["entries"][level]
        out = dict(agg=np.zeros(n_above, np.int32), mptr=np.zeros(n + 1, np.int32),
                   mem=np.zeros(n_above, np.int32), ptr=np.zeros(n + 1, np.int32),
                   col=np.zeros(nnz, np.int32), val=np.zeros(nnz, np.float32))
        self._check(self.lib.fcg_lp_hierarchy_level(self.h, ctx.h, int(level),
                                                    *[_ptr(out[k]) for k in ("agg", "mptr", "mem",
                                                                             "ptr", "col", "val")]),
                    "fcg_lp_hierarchy_level")
        return out

    def precondition(self, ctx: Context, r):
        """z = M(r): the network and the coarse-grid correction, as the solver applies it."""
        r = _f32(r)
        ctx._follow(r)
        z = _like(r)
        self._check(self.lib.fcg_lp_precondition(self.h, ctx.h, _ptr(r), _ptr(z)),
                    "fcg_lp_precondition")
        return z

    def coarse_correct(self, ctx: Context, r, z):
        """z + alpha P V(P^T (r - Ahat z)), the coarse-grid correction alone."""
        r, z = _f32(r), _f32(z)
        ctx._follow(r, z)
        out = _like(r)
        self._check(self.lib.fcg_lp_coarse_correct(self.h, ctx.h, _ptr(r), _ptr(z), _ptr(out)),
                    "fcg_lp_coarse_correct")
        return out

    # -- solver ---------------------------------------------------------------------
    def solve(self, ctx: Context, a, su, fi, sor: float, nsw: int) -> "FcgResult":
        """Learned-preconditioned flexible CG with the arguments of dpcg(fi,ifi)."""
        ctx._follow(a, su, fi)
        a, su = _host(a), _host(su)
        fi = fi.clone() if _is_torch(fi) else np.array(fi, dtype=np.float64)
        if _is_torch(su):
            import torch

            res = torch.zeros_like(su)
        else:
            res = np.zeros(ctx.n)
        resor = C.c_double(float("nan"))
        rep = _lib.SolveReport()
        it, fb = C.c_int(), C.c_int()
        rc = self.lib.fcg_fcg_learned(ctx.h, self.h, _ptr(a), _ptr(su), _ptr(fi), _ptr(res),
                                      float(sor), int(nsw), C.byref(resor), C.byref(rep),
                                      C.byref(it), C.byref(fb))
        ctx._check(rc, "fcg_fcg_learned")
        return FcgResult(fi, res, rep.res0, rep.resl, rep.iters, bool(rep.converged),
                         None if rep.iters == 0 else resor.value, rep.l2_rel, rep.seconds,
                         fcg_iters=it.value, fallback=bool(fb.value))


@dataclass
class FcgResult(SolveResult):
    fcg_iters: int = 0
    fallback: bool = False


# ---------------------------------------------------------------------------------
# Training data
# ---------------------------------------------------------------------------------
def diffusivity_field(m: Mesh, seed: int, lo: float = 0.1, hi: float = 10.0,
                      passes: int = 3) -> np.ndarray:
    """Per-cell diffusivity: log-uniform on [lo, hi], then `passes` Jacobi smoothing
    passes of log(diffusivity) over face neighbours (each cell becomes the mean of
    itself and its neighbours)."""
    g = np.log(lo) + (np.log(hi) - np.log(lo)) * uniform(seed, 9000, m.numCells, 0.0, 1.0)
    nin = m.numInnerFaces
    P, N = m.owner[:nin] - 1, m.neighbour[:nin] - 1
    cnt = np.ones(m.numCells)
    np.add.at(cnt, P, 1.0)
    np.add.at(cnt, N, 1.0)
    for _ in range(passes):
        s = g.copy()
        np.add.at(s, P, g[N])
        np.add.at(s, N, g[P])
        g = s / cnt
    return np.exp(g)


@dataclass
class TrainingSystem:
    mesh: Mesh
    ctx: Context
    a: np.ndarray
    su: np.ndarray
    scale: np.ndarray  # D^-1/2


def pressure_system(N: int, jitter: float, seed: int, variable: bool = True,
                    device: int = 0) -> TrainingSystem:
    """A pressure Poisson system on the N^3 jittered hex mesh: the laplacian with
    diffusivity `diffusivity_field` (or 1), RHS uniform[-1,1] * vol."""
    m = hex_mesh(N, jitter=jitter, seed=seed)
    ctx = Context(m, device)
    gam = diffusivity_field(m, seed) if variable else np.ones(m.numCells)
    su0 = uniform(seed, 0, m.numCells) * m.vol
    a, su = ctx.laplacian(-gam, np.zeros(m.numTotal), su0)
    io, ja, dg, _, _ = ctx.create_csr()
    return TrainingSystem(m, ctx, a, su, 1.0 / np.sqrt(a[dg - 1]))


def dpcg_pairs(sysm: TrainingSystem, ks, tight: float = 1e-13, nsw_max: int = 20000,
               device=None):
    """(r, e) pairs of the scaled system from DPCG iterates x_k (k sweeps from x = 0):
    r = D^-1/2 (su - A x_k), e = D^1/2 (x* - x_k), x* solved to `tight`.  FP32 arrays,
    or CUDA tensors when `device` is a torch device."""
    ctx, a, su, s = sysm.ctx, sysm.a, sysm.su, sysm.scale
    zero = np.zeros(ctx.n)
    xs = ctx.dpcg(a, su, zero, tight, nsw_max).fi
    out = []
    for k in ks:
        x = ctx.dpcg(a, su, zero, 0.0, int(k)).fi if k > 0 else zero
        r = (su - ctx.spmv(a, x)) * s
        e = (xs - x) / s
        r, e = r.astype(np.float32), e.astype(np.float32)
        if device is not None:
            import torch

            r, e = torch.from_numpy(r).to(device), torch.from_numpy(e).to(device)
        out.append((r, e))
    return out


def save_pairs(path: str, pairs, meta: dict | None = None):
    """One training-data shard: the (r, e) pairs of one system as FP32 arrays r[k], e[k]
    in an .npz, with optional scalar metadata (mesh size, seed, jitter, ...)."""
    def host(x):
        return x.detach().cpu().numpy() if _is_torch(x) else np.asarray(x, np.float32)

    r = np.stack([host(a) for a, _ in pairs]).astype(np.float32)
    e = np.stack([host(b) for _, b in pairs]).astype(np.float32)
    np.savez(path, r=r, e=e, **{f"meta_{k}": np.asarray(v) for k, v in (meta or {}).items()})


def load_pairs(path: str, device=None):
    """(pairs, meta) of a shard written by save_pairs; CUDA tensors when `device` is given."""
    d = np.load(path)
    pairs = []
    for r, e in zip(d["r"], d["e"]):
        if device is not None:
            import torch

            r, e = torch.from_numpy(r).to(device), torch.from_numpy(e).to(device)
        pairs.append((r, e))
    meta = {k[5:]: d[k].item() for k in d.files if k.startswith("meta_")}
    return pairs, meta


def train(lp: LearnedPreconditioner, systems, pairs, steps: int, lr: float = 1e-3, seed: int = 0,
          log_every: int = 0, log=print):
    """Adam on the pairs: `pairs[i]` is a list of (r, e) for `systems[i]`; each step
    takes one pair drawn uniformly (seeded).  Returns the per-step losses."""
    rng = np.random.default_rng(seed)
    flat = [(i, j) for i, ps in enumerate(pairs) for j in range(len(ps))]
    losses = np.zeros(steps)
    try:  # device copies of the matrices: switching systems is then a device copy
        import torch

        mats = [torch.from_numpy(np.ascontiguousarray(s.a)).cuda() for s in systems]
    except Exception:
        mats = [s.a for s in systems]
    cur = None
    t0 = time.perf_counter()
    for step in range(steps):
        i, j = flat[rng.integers(len(flat))]
        if cur != i:
            lp.set_matrix(systems[i].ctx, mats[i])
            cur = i
        r, e = pairs[i][j]
        losses[step] = lp.train_step(systems[i].ctx, r, e, lr)
        if log_every and (step + 1) % log_every == 0:
            log(f"step {step + 1}: mean loss {losses[step + 1 - log_every:step + 1].mean():.4f} "
                f"({time.perf_counter() - t0:.1f} s)")
    return losses


def train_default(path: str = DEFAULT_WEIGHTS, steps: int = 20000, n_pairs: int = 2000,
                  sizes=(64, 96), systems_per_size: int = 5, lr: float = 1e-3, seed: int = 7,
                  log=print):
    """The shipped checkpoint: `n_pairs` DPCG-iterate pairs from jittered meshes of the
    given sizes (jitter uniform on [0, 0.25] per mesh, smoothed log-uniform diffusivity
    on [0.1, 10]), Adam with rate `lr` for `steps` steps."""
    import torch

    dev = torch.device("cuda")
    per = n_pairs // (len(sizes) * systems_per_size)
    systems, pairs = [], []
    t0 = time.perf_counter()
    for si, N in enumerate(sizes):
        for j in range(systems_per_size):
            sd = seed * 1000 + si * 100 + j
            jit = 0.25 * uniform(sd, 77, 1, 0.0, 1.0)[0]
            sysm = pressure_system(N, jit, sd)
            conv = sysm.ctx.dpcg(sysm.a, sysm.su, np.zeros(sysm.ctx.n), 1e-8, 20000).iters
            ks = np.unique(np.round(np.linspace(0, conv, per)).astype(int))
            systems.append(sysm)
            pairs.append(dpcg_pairs(sysm, ks, device=dev))
            log(f"N={N} jitter={jit:.3f}: DPCG {conv} sweeps, {len(ks)} pairs "
                f"({time.perf_counter() - t0:.1f} s)")
    lp = LearnedPreconditioner(seed=seed)
    losses = train(lp, systems, pairs, steps, lr, seed, log_every=max(1, steps // 20), log=log)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    lp.save(path)
    return lp, losses


if __name__ == "__main__":  # python -m freecappuccino_gb300.learned [out_path] [steps]
    import sys

    out = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_WEIGHTS
    n_steps = int(sys.argv[2]) if len(sys.argv) > 2 else 20000
    t_start = time.perf_counter()
    train_default(out, steps=n_steps)
    print(f"saved {out} ({time.perf_counter() - t_start:.1f} s)")
