"""Learned preconditioner: a mesh graph network (3 message-passing layers of
width 32, FP32 weights, bf16 activations) evaluated and trained on the GPU
by the library's own kernels (csrc/gnn.cu) through the C ABI.

Training data are the solver's own (v_i, M^-1 v_i) pairs: the Arnoldi
vectors of an ILU(0)-preconditioned FGMRES restart cycle and their ILU(0)
corrections, collected over the Picard steps of transport problems with a
random velocity angle and diffusivity.  The default training loss is the
preconditioning residual ||A N(v) - v||^2 / ||v||^2 on those inputs; the
supervised loss against the ILU(0) correction is available
(loss="supervised" or "both") but a three-hop network fitted to ILU(0)'s
global corrections does not make FGMRES converge on its own.  The trained
network is the right preconditioner of FGMRES (precond="LEARNED"), with
ILU(0) as the fallback when a restart cycle stalls.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import FemGpuError, SSTransport, load

_vp = ctypes.c_void_p
WIDTH, LAYERS, NIN = 32, 3, 2


def param_shapes():
    s = [("We", (NIN, WIDTH)), ("be", (WIDTH,))]
    for l in range(LAYERS):
        s += [(f"Wh{l}", (WIDTH, WIDTH)), (f"W1{l}", (WIDTH, WIDTH)), (f"W2{l}", (WIDTH, WIDTH)),
              (f"b{l}", (WIDTH,))]
    return s + [("Wd", (WIDTH,)), ("bd", (1,))]


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation; residual-branch weights scaled by 0.3."""
    rng = np.random.default_rng(seed)
    out = []
    for name, sh in param_shapes():
        if name.startswith("W") and len(sh) == 2:
            sc = math.sqrt(2.0 / sh[0]) * (1.0 if name == "We" else 0.3)
            out.append(rng.normal(0.0, sc, sh).astype(np.float32).reshape(-1))
        elif name == "Wd":
            out.append(rng.normal(0.0, math.sqrt(1.0 / WIDTH), sh).astype(np.float32))
        else:
            out.append(np.zeros(int(np.prod(sh)), np.float32))
    return np.concatenate(out)


class MeshGNN:
    """Handle of a femgpu_gnn context."""

    def __init__(self, theta=None, bf16=True, seed=0):
        L = load()
        self._L = L
        self.nparams = L.femgpu_gnn_nparams()
        th = init_params(seed) if theta is None else np.ascontiguousarray(theta, np.float32)
        assert th.size == self.nparams
        h = _vp()
        rc = L.femgpu_gnn_create(ctypes.byref(h), 1 if bf16 else 0, th.ctypes.data_as(_vp))
        if rc:
            raise FemGpuError(rc, "gnn_create")
        self._h = h
        self.bf16 = bf16

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._L.femgpu_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where):
        if rc:
            raise FemGpuError(rc, where)

    def set_stream(self, stream_ptr):
        self._check(self._L.femgpu_gnn_set_stream(self._h, _vp(stream_ptr)), "set_stream")

    def params(self):
        th = np.zeros(self.nparams, np.float32)
        self._check(self._L.femgpu_gnn_get_params(self._h, th.ctypes.data_as(_vp)), "get_params")
        return th

    def set_params(self, theta):
        th = np.ascontiguousarray(theta, np.float32)
        self._check(self._L.femgpu_gnn_set_params(self._h, th.ctypes.data_as(_vp)), "set_params")

    def grad(self):
        g = np.zeros(self.nparams, np.float32)
        self._check(self._L.femgpu_gnn_get_grad(self._h, g.ctypes.data_as(_vp)), "get_grad")
        return g

    def attach_csr(self, IA, JA, AA):
        IA = np.ascontiguousarray(IA, np.int32)
        JA = np.ascontiguousarray(JA, np.int32)
        AA = np.ascontiguousarray(AA, np.float64)
        self.n = len(IA) - 1
        self._check(self._L.femgpu_gnn_attach_csr(self._h, self.n, IA.ctypes.data_as(_vp),
                                                  JA.ctypes.data_as(_vp), AA.ctypes.data_as(_vp)), "attach")

    def attach_transport(self, T: SSTransport):
        IA, JA, AA = T.csr_dev()
        self.n = T.neq
        self._check(self._L.femgpu_gnn_attach_csr_dev(self._h, T.neq, T.nnzero, _vp(IA), _vp(JA), _vp(AA)),
                    "attach")

    def apply(self, r):
        r = np.ascontiguousarray(r[: self.n], np.float64)
        z = np.zeros(self.n)
        self._check(self._L.femgpu_gnn_apply(self._h, r.ctypes.data_as(_vp), z.ctypes.data_as(_vp)), "apply")
        return z

    def apply_dev(self, r_ptr, z_ptr):
        """z = N(r) on device buffers (FP64, n entries each), on the context's stream."""
        self._check(self._L.femgpu_gnn_apply_dev(self._h, _vp(r_ptr), _vp(z_ptr)), "apply_dev")

    def loss_grad(self, r, t):
        """Host-buffer forward + backward: (loss, grad, z)."""
        r = np.ascontiguousarray(r[: self.n], np.float64)
        t = np.ascontiguousarray(t[: self.n], np.float64)
        loss = ctypes.c_double(0.0)
        g = np.zeros(self.nparams, np.float32)
        z = np.zeros(self.n)
        self._check(self._L.femgpu_gnn_loss_grad(self._h, r.ctypes.data_as(_vp), t.ctypes.data_as(_vp),
                                                 ctypes.byref(loss), g.ctypes.data_as(_vp),
                                                 z.ctypes.data_as(_vp)), "loss_grad")
        return loss.value, g, z

    def loss_grad_dev(self, r_ptr, t_ptr, z_ptr, accumulate, want_loss=False):
        loss = ctypes.c_double(0.0)
        self._check(self._L.femgpu_gnn_loss_grad_dev(self._h, _vp(r_ptr), _vp(t_ptr), _vp(z_ptr),
                                                     1 if accumulate else 0,
                                                     ctypes.byref(loss) if want_loss else None), "loss_grad")
        return loss.value if want_loss else None

    LOSSES = {"supervised": 0, "residual": 1, "both": 2}

    def set_loss(self, kind):
        """Training loss: "supervised" (ILU(0) target), "residual"
        (||A z - r||) or "both"."""
        self._check(self._L.femgpu_gnn_set_loss(self._h, self.LOSSES[kind]), "set_loss")

    def adam(self, lr, gscale=1.0):
        self._check(self._L.femgpu_gnn_adam_step(self._h, float(lr), float(gscale)), "adam")


# ------------------------------------------------------------------ data
def transport_problem(nx, ny, angle, k, seed):
    """A rotated-velocity transport problem on a perturbed nx x ny mesh."""
    from .mesh import rotated_problem, structured_mesh
    m = structured_mesh(nx, ny, perturb=0.2, seed=seed)
    return m, rotated_problem(m, angle, k)


def sample_problems(count, sizes, seed):
    """count (nx, angle, k, seed) draws: nx from sizes, angle U[0, 2pi),
    k log-uniform in [1e-6, 1e-2]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        nx = int(rng.choice(sizes))
        out.append((nx, float(rng.uniform(0.0, 2.0 * math.pi)), float(10.0 ** rng.uniform(-6.0, -2.0)),
                    int(rng.integers(1, 1 << 30))))
    return out


class PairSet:
    """(residual, ILU(0) correction) pairs of one problem, on the device."""

    def __init__(self, T, V, Z):
        self.T, self.V, self.Z = T, V, Z

    @property
    def count(self):
        return self.V.shape[0]


def collect_pairs(spec, picard_steps=2, kmax=50):
    """Run ILU(0)-FGMRES(kmax) Picard steps of a problem and keep the first
    restart cycle's Arnoldi vectors and their ILU(0) corrections of each
    step.  Returns a PairSet (torch tensors [pairs, neq] on the GPU)."""
    import torch
    nx, angle, k, seed = spec
    m, p = transport_problem(nx, nx, angle, k, seed)
    T = SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", kmax=kmax, lmax=1,
                                 tol=1e-12, solver="FGMRES")
    Vs, Zs = [], []
    for _ in range(picard_steps):
        T.build_dev()
        T.precond_setup_dev(1)
        try:
            T.solve_dev()
        except FemGpuError as e:
            if e.code != -5:
                raise
        V = torch.zeros(kmax, T.neq, dtype=torch.float64, device="cuda")
        Z = torch.zeros_like(V)
        torch.cuda.synchronize()
        c = T.krylov_pairs(V.data_ptr(), Z.data_ptr(), T.neq, kmax)
        Vs.append(V[:c])
        Zs.append(Z[:c])
    return PairSet(T, torch.cat(Vs), torch.cat(Zs))


def train(gnn: MeshGNN, sets, epochs=4, lr=2e-3, batch=8, seed=0, log=None, loss="residual"):
    """Adam on the mean loss over minibatches of pairs drawn from one problem
    at a time; the learning rate decays linearly to lr/10 over the run.
    Returns the per-epoch mean loss (sampled every 20 steps)."""
    import torch
    rng = np.random.default_rng(seed)
    gnn.set_loss(loss)
    nsteps = epochs * sum((s.count + batch - 1) // batch for s in sets)
    zbuf = {}
    hist = []
    step = 0
    for ep in range(epochs):
        jobs = []
        for si, s in enumerate(sets):
            idx = rng.permutation(s.count)
            for b in range(0, len(idx), batch):
                jobs.append((si, idx[b:b + batch]))
        rng.shuffle(jobs)
        tot, cnt = 0.0, 0
        for si, ids in jobs:
            s = sets[si]
            gnn.attach_transport(s.T)
            z = zbuf.get(s.T.neq)
            if z is None:
                z = zbuf[s.T.neq] = torch.zeros(s.T.neq, dtype=torch.float64, device="cuda")
            for q, i in enumerate(ids):
                want = (q == len(ids) - 1) and (step % 20 == 0)
                L = gnn.loss_grad_dev(s.V[i].data_ptr(), s.Z[i].data_ptr(), z.data_ptr(), q > 0, want)
                if want:
                    tot += L
                    cnt += 1
            gnn.adam(lr * (1.0 - 0.9 * step / max(nsteps, 1)), 1.0 / len(ids))
            step += 1
        torch.cuda.synchronize()
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return hist


def evaluate(spec, gnn=None, kmax=50, tol=1e-8, lmax=400, stall_ratio=0.9, precond=None, amg=None):
    """FGMRES(kmax) on one problem's first Picard system with the learned
    preconditioner (gnn given), ILU(0) or none: (iterations, seconds to
    solution, true relative residual, fell back: 0 no, 1 to ILU(0), 2 to the
    AMG context amg when one is given)."""
    import torch
    nx, angle, k, seed = spec
    m, p = transport_problem(nx, nx, angle, k, seed)
    pc = precond or ("LEARNED" if gnn is not None else "ILU0")
    T = SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond=pc, kmax=kmax, lmax=lmax,
                                 tol=tol, solver="FGMRES", stall_ratio=stall_ratio)
    if gnn is not None and pc == "LEARNED":
        T.set_learned(gnn)
        if amg is not None:
            T.set_amg(amg)
    T.build_dev()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    T.precond_setup_dev(1)
    it = T.solve_dev(raise_on_nonconvergence=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    rel = T.true_residual()
    fell = pc == "LEARNED" and T.fell_back()
    T.close()
    return dict(iters=it, seconds=dt, rel=rel, converged=rel <= tol * 1.0001, fell_back=fell)


def grid_csr(nx, seed=0):
    """A 5-point upwinded advection-diffusion pattern on an nx x nx grid
    (CSR, columns ascending in each row)."""
    n = nx * nx
    i = np.arange(n)
    x, y = i % nx, i // nx
    cols = [i, i - 1, i + 1, i - nx, i + nx]
    ok = [x >= 0, x > 0, x < nx - 1, y > 0, y < nx - 1]
    vals = [np.full(n, 4.4), np.full(n, -1.3), np.full(n, -0.7), np.full(n, -1.2), np.full(n, -0.8)]
    nnz_row = np.sum(ok, axis=0)
    IA = np.zeros(n + 1, np.int64)
    IA[1:] = np.cumsum(nnz_row)
    JA = np.concatenate([c[m] for c, m in zip(cols, ok)])
    AA = np.concatenate([v[m] for v, m in zip(vals, ok)])
    order = np.lexsort((JA, np.concatenate([i[m] for m in ok])))
    return IA.astype(np.int32), JA[order].astype(np.int32), AA[order]


def time_apply(nx, reps=20, warmup=3):
    """CUDA-event time of one network application (bf16 activations) on the
    nx x nx grid graph, inputs resident on the device; returns ms."""
    import torch
    IA, JA, AA = grid_csr(nx)
    net = MeshGNN(init_params(7), bf16=True)
    stream = torch.cuda.Stream()            # a stream of its own: the context keeps its stream when given NULL
    net.set_stream(stream.cuda_stream)
    net.attach_csr(IA, JA, AA)
    r = torch.randn(net.n, dtype=torch.float64, device="cuda")
    z = torch.empty_like(r)
    torch.cuda.synchronize()
    for _ in range(warmup):
        net.apply_dev(r.data_ptr(), z.data_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        net.apply_dev(r.data_ptr(), z.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    net.close()
    return e0.elapsed_time(e1) / reps


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time one learned-preconditioner application on a grid graph")
    ap.add_argument("--nx", type=int, default=1024)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args()
    print(json.dumps({"nodes": a.nx * a.nx, "ms_per_apply": time_apply(a.nx, a.reps)}))
