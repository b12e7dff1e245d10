"""numpy oracle of the learned preconditioner (learned.cu in libfcgpu.so).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA network kernels; only ``tests/``
may import it.  The learned preconditioner has no counterpart in the reference, so
there is nothing of the reference to pin it to: this module restates the network as
learned.cu documents it (features, forward, loss, straight-through backward, Adam) and
is itself checked against central finite differences of its own FP64 forward
(tests/test_learned.py).

``emulate=True`` rounds at the same points as the CUDA forward: activations h and
aggregates Ahat h to BF16 (round to nearest even), the layer weights W_l to BF16; the
backward then treats the roundings as identities and uses the FP32 master weights, as
the CUDA backward does.  ``emulate=False`` is the plain FP64 function.
"""
from __future__ import annotations

import numpy as np

C, L, F = 32, 6, 6
LAYER = 2 * C * C + C
P = C * F + C + L * LAYER + C + 1


def bf16(x) -> np.ndarray:
    """Round to BF16 (nearest, ties to even), returned as float64."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    assert w.size == P
    o = 0
    W_in = w[o:o + C * F].reshape(C, F); o += C * F
    b_in = w[o:o + C]; o += C
    layers = []
    for _ in range(L):
        Wl = w[o:o + 2 * C * C].reshape(C, 2 * C); o += 2 * C * C
        bl = w[o:o + C]; o += C
        layers.append((Wl, bl))
    w_out = w[o:o + C]; o += C
    b_out = w[o]
    return W_in, b_in, layers, w_out, b_out


def pack(W_in, b_in, layers, w_out, b_out) -> np.ndarray:
    parts = [W_in.ravel(), b_in]
    for Wl, bl in layers:
        parts += [Wl.ravel(), bl]
    parts += [w_out, np.atleast_1d(b_out)]
    return np.concatenate(parts)


class ScaledMatrix:
    """Ahat = D^-1/2 A D^-1/2 from the reference's 1-based CSR, values rounded to FP32 as
    the CUDA fill does ((a_ij s_i) s_j in FP64, then FP32)."""

    def __init__(self, ioffset, ja, diag, a):
        io = np.asarray(ioffset) - 1
        self.n = len(io) - 1
        self.rows = np.repeat(np.arange(self.n), np.diff(io))
        self.cols = np.asarray(ja) - 1
        a = np.asarray(a, dtype=np.float64)
        self.s = 1.0 / np.sqrt(a[np.asarray(diag) - 1])
        self.val = (a * self.s[self.rows] * self.s[self.cols]).astype(np.float32).astype(np.float64)

    def matmul(self, X):
        """Ahat X for X of shape (n, k)."""
        out = np.zeros((self.n,) + X.shape[1:])
        np.add.at(out, self.rows, self.val[:, None] * X[self.cols])
        return out

    def rmatmul(self, X):
        """Ahat^T X."""
        out = np.zeros((self.n,) + X.shape[1:])
        np.add.at(out, self.cols, self.val[:, None] * X[self.rows])
        return out


def features(m, s) -> np.ndarray:
    """Static per-cell inputs 1..5 (column 0, the residual, is left 0): log(a_PP /
    vol^1/3) - log 6, log(vol / mean vol), sum|S_x,y,z| over the cell's faces divided by
    2 vol^2/3, minus 1.  `m` has the reference's face arrays (owner/neighbour 1-based)."""
    n, nin, nf = m.numCells, m.numInnerFaces, m.numFaces
    vol = np.asarray(m.vol, dtype=np.float64)
    d = 1.0 / (np.asarray(s) ** 2)
    h = np.cbrt(vol)
    own = np.asarray(m.owner[:nf]) - 1
    nb = np.asarray(m.neighbour[:nin]) - 1
    out = np.zeros((n, F))
    out[:, 1] = np.log(d / h) - np.log(6.0)
    out[:, 2] = np.log(vol / (vol.sum() / n))
    for k, ar in enumerate((m.arx, m.ary, m.arz)):
        a = np.abs(np.asarray(ar[:nf], dtype=np.float64))
        acc = np.zeros(n)
        np.add.at(acc, own, a)
        np.add.at(acc, nb, a[:nin])
        out[:, 3 + k] = acc / (2.0 * h * h) - 1.0
    return out.astype(np.float32).astype(np.float64)


def forward(A: ScaledMatrix, feat, r, w, emulate: bool = True):
    """Returns (z, cache): z = r + rms (w_out . h_L + b_out) and what the backward needs
    (y = z / rms, the normalised output)."""
    W_in, b_in, layers, w_out, b_out = unpack(w)
    rd = lambda x: bf16(x) if emulate else x
    r = np.asarray(r, dtype=np.float64)
    rms = np.sqrt(np.dot(r, r) / len(r))
    if rms == 0:
        rms = 1.0
    f = np.array(feat, dtype=np.float64)
    f[:, 0] = r / rms
    z0 = f @ W_in.T + b_in
    h = rd(np.maximum(z0, 0.0))
    hs, xs, zs = [h], [], []
    for Wl, bl in layers:
        mb = rd(A.matmul(h))
        x = np.concatenate([h, mb], axis=1)
        zl = x @ rd(Wl).T + bl
        h = rd(h + np.maximum(zl, 0.0))
        hs.append(h)
        xs.append(x)
        zs.append(zl)
    y = f[:, 0] + h @ w_out + b_out
    return rms * y, dict(rms=rms, f=f, z0=z0, hs=hs, xs=xs, zs=zs, y=y)


def loss_grad(A: ScaledMatrix, feat, r, e, w, emulate: bool = True, kind: str = "energy",
              correct=None):
    """Loss of the normalised output d = y - t, t = e/rms, and its gradient
    (straight-through roundings, Ahat symmetric):
      energy:   d.Ahat d / t.Ahat t,        d loss/dy = 2 Ahat d / t.Ahat t
      residual: |Ahat d|^2 / |Ahat t|^2,    d loss/dy = 2 Ahat Ahat d / |Ahat t|^2
      cycle:    the energy form of y_c = correct(r/rms, y) = y + alpha P V P^T (r/rms -
                Ahat y), the coarse-grid correction after the network (a callable, e.g.
                multilevel_oracle.Cycle.correct): d = y_c - t and, V being symmetric,
                d loss/dy = u - Ahat correct(u, 0), u = 2 Ahat d / t.Ahat t"""
    W_in, b_in, layers, w_out, b_out = unpack(w)
    z, c = forward(A, feat, r, w, emulate)
    t = np.asarray(e, dtype=np.float64) / c["rms"]
    y = c["y"]
    if kind == "cycle":
        y = correct(c["f"][:, 0], y)
    d = y - t
    Ad = A.matmul(d[:, None])[:, 0]
    At = A.matmul(t[:, None])[:, 0]
    if kind in ("energy", "cycle"):
        den = np.dot(t, At)
        loss = np.dot(d, Ad) / den
        dy = 2.0 * Ad / den
        if kind == "cycle":
            dy = dy - A.matmul(correct(dy, np.zeros_like(dy))[:, None])[:, 0]
    else:
        den = np.dot(At, At)
        loss = np.dot(Ad, Ad) / den
        dy = 2.0 * A.matmul(Ad[:, None])[:, 0] / den
    g_wout = c["hs"][-1].T @ dy
    g_bout = dy.sum()
    dh = np.outer(dy, w_out)
    g_layers = [None] * L
    for l in range(L - 1, -1, -1):
        Wl, bl = layers[l]
        dz = dh * (c["zs"][l] > 0)
        gW = dz.T @ c["xs"][l]
        gb = dz.sum(axis=0)
        dx = dz @ Wl
        dh = dh + dx[:, :C] + A.rmatmul(dx[:, C:])
        g_layers[l] = (gW, gb)
    dz0 = dh * (c["z0"] > 0)
    g_Win = dz0.T @ c["f"]
    g_bin = dz0.sum(axis=0)
    return loss, pack(g_Win, g_bin, g_layers, g_wout, g_bout)


def adam(w, m, v, g, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) in FP32 as the CUDA kernel orders it."""
    f = np.float32
    w, m, v, g = (np.asarray(x, dtype=f) for x in (w, m, v, g))
    m = f(b1) * m + (f(1) - f(b1)) * g
    v = f(b2) * v + (f(1) - f(b2)) * g * g
    c1 = f(1) - f(b1) ** f(step)
    c2 = f(1) - f(b2) ** f(step)
    w = w - f(lr) * (m / c1) / (np.sqrt(v / c2) + f(eps))
    return w, m, v
