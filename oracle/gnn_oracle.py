"""Test infrastructure only -- CPU oracle of the learned preconditioner.

The reference has no learned component; this is a plain numpy restatement of
this project's own mesh graph network (fem_codes_gb300/csrc/gnn.cu), used by
the tests to check the CUDA forward pass, the hand-written backward pass and
the Adam step.  Activations may be rounded to bfloat16 at the same points as
the device kernels store them (round to nearest even).

Network (width W = 32, L = 3 message-passing layers) on the graph of a CSR
matrix A (pattern structurally symmetric, diagonal present):
  s      = sqrt(mean(r^2)),  r^ = r / s,  dbar = mean(|a_ii|)
  x_i    = [r^_i, r^_i dbar / a_ii]
  h0_i   = relu(We^T x_i + be)
  layer l:  m1_i = sum_{j != i} (a_ij / a_ii) h_j      (wA, row i)
            m2_i = sum_{j != i} (a_ji / a_jj) h_j      (wT, row i)
            u_i  = Wh^T h_i + W1^T m1_i + W2^T m2_i + b
            h'_i = h_i + relu(u_i)
  y_i    = Wd . h_L,i + bd
  z_i    = s y_i dbar / a_ii
Loss against a target correction t (the ILU(0)-preconditioned residual):
  L = sum (z - t)^2 / sum t^2.
"""
from __future__ import annotations

import numpy as np

WIDTH = 32
LAYERS = 3
NIN = 2


def param_shapes(width=WIDTH, layers=LAYERS):
    s = [("We", (NIN, width)), ("be", (width,))]
    for l in range(layers):
        s += [(f"Wh{l}", (width, width)), (f"W1{l}", (width, width)), (f"W2{l}", (width, width)),
              (f"b{l}", (width,))]
    s += [("Wd", (width,)), ("bd", (1,))]
    return s


def nparams(width=WIDTH, layers=LAYERS):
    return sum(int(np.prod(sh)) for _, sh in param_shapes(width, layers))


def unpack(theta, width=WIDTH, layers=LAYERS):
    out, o = {}, 0
    for name, sh in param_shapes(width, layers):
        k = int(np.prod(sh))
        out[name] = theta[o:o + k].reshape(sh)
        o += k
    return out


def pack(p, width=WIDTH, layers=LAYERS, dt=np.float32):
    return np.concatenate([np.asarray(p[n], dt).reshape(-1) for n, _ in param_shapes(width, layers)])


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    x = np.asarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def graph(IA, JA, AA):
    """(rows, cols, wA, wT, d) over the off-diagonal entries of a CSR matrix."""
    n = len(IA) - 1
    rows = np.repeat(np.arange(n), np.diff(IA))
    cols = np.asarray(JA)
    vals = np.asarray(AA[: len(JA)], np.float64)
    d = np.zeros(n)
    dm = rows == cols
    d[rows[dm]] = vals[dm]
    off = ~dm
    r, c, v = rows[off], cols[off], vals[off]
    wA = (v / d[r]).astype(np.float32)
    # a_ji / a_jj for each (i, j): look up the transposed entry
    key = r.astype(np.int64) * n + c
    tkey = c.astype(np.int64) * n + r
    order = np.argsort(key)
    pos = order[np.searchsorted(key[order], tkey)]
    wT = wA[pos]
    return r, c, wA, wT, d


def _spmm(n, r, c, w, h):
    out = np.zeros((n, h.shape[1]), np.float64)
    np.add.at(out, r, w[:, None].astype(np.float64) * h[c].astype(np.float64))
    return out.astype(h.dtype)


def forward(theta, g, rvec, act_bf16=True, width=WIDTH, layers=LAYERS, dt=np.float32):
    """Returns (z, cache).  dt=np.float64 (with act_bf16=False) evaluates the
    same network in double precision, for finite-difference checks."""
    p = unpack(np.asarray(theta, dt), width, layers)
    rr, cc, wA, wT, d = g
    wA, wT = wA.astype(dt), wT.astype(dt)
    n = len(d)
    q = bf16 if act_bf16 else (lambda a: np.asarray(a, dt))
    r = np.asarray(rvec[:n], np.float64)
    s = float(np.sqrt(np.mean(r * r)))
    s = s if s > 0 else 1.0
    dbar = float(np.mean(np.abs(d)))
    rh = (r / s).astype(dt)
    x = np.stack([rh, (rh * dt(dbar) / d.astype(dt)).astype(dt)], 1)
    pre0 = x @ p["We"] + p["be"]
    h = [q(np.maximum(pre0, 0))]
    m1s, m2s, us = [], [], []
    for l in range(layers):
        m1 = q(_spmm(n, rr, cc, wA, h[-1]))
        m2 = q(_spmm(n, rr, cc, wT, h[-1]))
        u = h[-1] @ p[f"Wh{l}"] + m1 @ p[f"W1{l}"] + m2 @ p[f"W2{l}"] + p[f"b{l}"]
        h.append(q(h[-1] + np.maximum(u, 0)))
        m1s.append(m1); m2s.append(m2); us.append(u)
    y = h[-1] @ p["Wd"] + p["bd"][0]
    z = (s * y.astype(np.float64) * dbar / d)
    cache = dict(p=p, x=x, pre0=pre0, h=h, m1=m1s, m2=m2s, u=us, s=s, dbar=dbar, g=g)
    return z, cache


def amul(g, z):
    """A z with A = diag(d) (I + W), W the off-diagonal wA (as the device
    graph holds it)."""
    rr, cc, wA, wT, d = g
    s = np.asarray(z, np.float64).copy()
    np.add.at(s, rr, wA.astype(np.float64) * z[cc])
    return d * s


def atmul(g, y):
    """A^T y for the same A."""
    rr, cc, wA, wT, d = g
    s = d * y
    np.add.at(s, cc, wA.astype(np.float64) * d[rr] * y[rr])
    return s


def loss_and_grad(theta, g, rvec, target, act_bf16=True, width=WIDTH, layers=LAYERS, dt=np.float32,
                  kind=0):
    """(L, dL/dtheta, z) by the hand-derived backward pass.  kind 0:
    ||z - t||^2/||t||^2, 1: ||A z - r||^2/||r||^2, 2: both summed."""
    z, c = forward(theta, g, rvec, act_bf16, width, layers, dt)
    p, h = c["p"], c["h"]
    rr, cc, wA, wT, d = g
    n = len(d)
    t = np.asarray(target[:n], np.float64)
    r = np.asarray(rvec[:n], np.float64)
    L, gz = 0.0, np.zeros(n)
    if kind != 1:
        T2 = float(np.sum(t * t))
        L += float(np.sum((z - t) ** 2) / T2)
        gz += 2.0 * (z - t) / T2
    if kind != 0:
        res = amul(g, z) - r
        R2 = float(np.sum(r * r))
        L += float(np.sum(res * res) / R2)
        gz += 2.0 * atmul(g, res) / R2
    gy = (gz * c["s"] * c["dbar"] / d).astype(dt)
    wA, wT = wA.astype(dt), wT.astype(dt)
    gr = {k: np.zeros_like(v) for k, v in p.items()}
    gr["Wd"] = h[-1].T @ gy
    gr["bd"] = np.array([gy.sum()], dt)
    gh = np.outer(gy, p["Wd"]).astype(dt)
    for l in reversed(range(layers)):
        gu = gh * (c["u"][l] > 0)
        gr[f"Wh{l}"] = h[l].T @ gu
        gr[f"W1{l}"] = c["m1"][l].T @ gu
        gr[f"W2{l}"] = c["m2"][l].T @ gu
        gr[f"b{l}"] = gu.sum(0)
        gm1 = gu @ p[f"W1{l}"].T
        gm2 = gu @ p[f"W2{l}"].T
        # transpose of m1_i = sum wA h_j, m2_i = sum wT h_j
        back = _spmm(n, cc, rr, wA, gm1) + _spmm(n, cc, rr, wT, gm2)
        gh = gh + gu @ p[f"Wh{l}"].T + back
    gpre = gh * (c["pre0"] > 0)
    gr["We"] = c["x"].T @ gpre
    gr["be"] = gpre.sum(0)
    return L, pack(gr, width, layers, dt), z


def init(seed=0, width=WIDTH, layers=LAYERS):
    """He-style initialisation scaled so the residual branches start small."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, sh in param_shapes(width, layers):
        if name.startswith("W") and len(sh) == 2:
            fan = sh[0]
            scale = np.sqrt(2.0 / fan) * (1.0 if name == "We" else 0.3)
            p[name] = rng.normal(0, scale, sh).astype(np.float32)
        else:
            p[name] = np.zeros(sh, np.float32)
    p["Wd"] = rng.normal(0, np.sqrt(1.0 / width), (width,)).astype(np.float32)
    return pack(p, width, layers)


def adam(theta, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (in place on theta, m, v); step counts from 1."""
    m[:] = b1 * m + (1 - b1) * grad
    v[:] = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    theta[:] = theta - lr * mh / (np.sqrt(vh) + eps)
    return theta
