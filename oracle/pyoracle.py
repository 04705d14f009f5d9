"""Test infrastructure only: ctypes access to the CPU oracle (liboracle.so,
built from oracle/*_oracle.c by ``make -C oracle``).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None


_libfast = None


def build(name: str = "liboracle.so") -> str:
    subprocess.run(["make", "-s", "-C", HERE, name], check=True)
    return os.path.join(HERE, name)


def lib(fast: bool = False) -> ctypes.CDLL:
    """The oracle library: liboracle.so (bit-stable FP64, the parity checker)
    or, with fast=True, liboracle_fast.so (the same sources -Ofast, as the
    reference's Makefiles build it; the timed CPU baseline)."""
    global _lib, _libfast
    if (_libfast if fast else _lib) is None:
        name = "liboracle_fast.so" if fast else "liboracle.so"
        path = os.path.join(HERE, name)
        srcs = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".c", ".h"))
                and not f.startswith("ref_")]
        if not os.path.exists(path) or any(os.path.getmtime(path) < os.path.getmtime(f) for f in srcs):
            build(name)
        L = ctypes.CDLL(path)
        L.orc_transport_run.restype = ctypes.c_int
        L.orc_transport_run.argtypes = [
            ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_double, ctypes.c_double,
            _dp, _dp, _dp,
            ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
            ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
            ctypes.c_double, _ip, _ip, _ip, _ip, _ip, _ip, _ip,
            _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        L.orc_fill_lm.restype = ctypes.c_int
        L.orc_fill_lm.argtypes = [ctypes.c_int, _ip, ctypes.c_int, _ip, _ip, _ip]
        L.orc_csr_pattern.restype = ctypes.c_int
        L.orc_csr_pattern.argtypes = [ctypes.c_int, ctypes.c_int, _ip, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
        L.orc_symrcm.restype = None
        L.orc_symrcm.argtypes = [ctypes.c_int, _ip, _ip, _ip]
        L.orc_reorder_csr.restype = ctypes.c_int
        L.orc_reorder_csr.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _ip, _ip, ctypes.c_int,
                                      _ip, ctypes.c_int, _ip]
        L.orc_ede_pattern.restype = ctypes.c_int
        L.orc_ede_pattern.argtypes = [ctypes.c_int, ctypes.c_int, _ip, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
        L.orc_csrmv.restype = None
        L.orc_csrmv.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, _dp]
        L.orc_ebemv.restype = None
        L.orc_ebemv.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _dp]
        L.orc_edemv.restype = None
        L.orc_edemv.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _dp]
        L.orc_ilu0_factor.restype = ctypes.c_int
        L.orc_ilu0_factor.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, _dp]
        L.orc_ilu0_apply.restype = None
        L.orc_ilu0_apply.argtypes = [ctypes.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
        L.orc_csr_gmres.restype = ctypes.c_int
        L.orc_csr_gmres.argtypes = [ctypes.c_int, _ip, _ip, _dp, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, _dp, _dp]
        L.orc_amg_vcycle.restype = ctypes.c_int
        L.orc_amg_vcycle.argtypes = [ctypes.c_int, _ip, _ip, _ip, _dp, _ip, ctypes.c_double, ctypes.c_int,
                                     _dp, _dp]
        L.orc_amg_gmres.restype = ctypes.c_int
        L.orc_amg_gmres.argtypes = [ctypes.c_int, _ip, _ip, _ip, _dp, _ip, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp]
        L.orc_ddot.restype = ctypes.c_double
        L.orc_ddot.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_get_times.restype = None
        L.orc_get_times.argtypes = [_dp]
        L.orc_get_step_times.restype = None
        L.orc_get_step_times.argtypes = [_dp, ctypes.c_int]
        L.orc_set_refine.restype = None
        L.orc_set_refine.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_set_refine_window.restype = None
        L.orc_set_refine_window.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_get_refine.restype = None
        L.orc_get_refine.argtypes = [_dp, _ip, ctypes.c_int]
        if fast:
            _libfast = L
        else:
            _lib = L
    return _libfast if fast else _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def run_transport(x, y, node_type, vert, k, gamma, beta, fsrc, upresc, scheme="CSR",
                  reord="NOT", precond="ILU0", shock="CAU", hshock="2sqrtArea", outflow="NOT",
                  kmax=30, lmax=1000, tol=1e-8, npicard=3, nonlin_tol=0.0, Pin=None, fast=False,
                  refine_to=0.0, refine_tol=1e-12, refine_max=40, refine_from=0, refine_budget_s=0.0):
    """Full steady-transport run; same outputs as the reference harness.
    fast: the -Ofast build.  refine_to > 0: the to-solution variant (every
    Picard solve from step refine_from on refined with the reference's pgmres
    until the true relative residual is <= refine_to, the Picard loop ending
    once refine_budget_s seconds went into refined steps (0: no bound));
    out["refine"] then holds, per Picard step, the final true residual (-1 for
    unrefined steps) and the refinement rounds."""
    L = lib(fast)
    L.orc_set_refine(float(refine_to), float(refine_tol), int(refine_max))
    L.orc_set_refine_window(int(refine_from), float(refine_budget_s))
    nn, ne = len(x), len(vert)
    node_type = _c(node_type, np.int32)
    neq_ub = int((node_type >= 1).sum())
    nnz_ub = 9 * ne + 1
    info = np.zeros(4, np.int32)
    node_id = np.zeros(nn, np.int32)
    etype = np.zeros(ne, np.int32)
    IA = np.zeros(neq_ub + 1, np.int32)
    JA = np.zeros(max(nnz_ub, 6 * ne + 2), np.int32)
    sbe = np.zeros(9 * ne, np.int32)
    order = np.zeros(3 * ne, np.int32)
    Afirst = np.zeros(max(9 * ne, 4 * (3 * ne + 1), nnz_ub))
    Ffirst = np.zeros(neq_ub + 1)
    Fprec = np.zeros(neq_ub + 1)
    if Pin is None:
        Pin = np.random.default_rng(7).uniform(-1.0, 1.0, neq_ub + 1)
    Pin = _c(Pin, np.float64)
    Qmv = np.zeros(neq_ub + 1)
    Zpc = np.zeros(neq_ub + 1)
    uhist = np.zeros(npicard * (neq_ub + 1))
    iters = np.zeros(npicard, np.int32)
    nit = L.orc_transport_run(
        nn, _c(x, np.float64), _c(y, np.float64), node_type, ne, _c(vert, np.int32).reshape(-1),
        float(k), float(gamma), _c(beta, np.float64).reshape(-1), _c(fsrc, np.float64).reshape(-1),
        _c(upresc, np.float64), scheme.encode(), reord.encode(), precond.encode(), shock.encode(),
        hshock.encode(), outflow.encode(), kmax, lmax, tol, npicard, nonlin_tol,
        info, node_id, etype, IA, JA, sbe, order, Afirst, Ffirst, Fprec, Pin, Qmv, Zpc,
        uhist, iters)
    L.orc_set_refine(0.0, 0.0, 0)
    if nit < 0:
        raise RuntimeError(f"oracle run failed ({nit})")
    neq, nnz, nedge, bw = (int(v) for v in info)
    out = dict(neq=neq, nnzero=nnz, nedge=nedge, bandwidth=bw, npicard_run=nit,
               node_id=node_id, etype=etype, Ffirst=Ffirst, Fprec=Fprec, Pin=Pin, Qmv=Qmv,
               Zpc=Zpc, uhist=uhist[: nit * (neq + 1)].reshape(nit, neq + 1), iters=iters[:nit])
    if refine_to > 0:
        res = np.zeros(max(nit, 1))
        rounds = np.zeros(max(nit, 1), np.int32)
        L.orc_get_refine(res, rounds, max(nit, 1))
        out["refine"] = {"true_rel_residual": res[:nit], "rounds": rounds[:nit]}
    if scheme.upper() == "CSR":
        out.update(IA=IA[: neq + 1], JA=JA[:nnz], sbe=sbe.reshape(ne, 9), Afirst=Afirst[: nnz + 1])
    elif scheme.upper() == "EDE":
        out.update(lm2=JA[: 2 * nedge].reshape(nedge, 2), sbe=sbe[: 3 * ne].reshape(ne, 3),
                   order=order.reshape(ne, 3), Afirst=Afirst[: 4 * (nedge + 1)].reshape(nedge + 1, 4))
    else:
        out.update(Afirst=Afirst[: 9 * ne].reshape(ne, 9))
    return out


def _blk_lib():
    L = lib()
    if not hasattr(L, "_blk_ready"):
        L.orc_fill_lm_blk.restype = None
        L.orc_fill_lm_blk.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.c_int, _ip]
        L.orc_ebemv_blk.restype = None
        L.orc_ebemv_blk.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _dp]
        L.orc_blockdiag_setup.restype = None
        L.orc_blockdiag_setup.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip,
                                          _dp, _dp, _dp, ctypes.c_void_p]
        L.orc_blockdiag_apply.restype = None
        L.orc_blockdiag_apply.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _dp]
        L.orc_ebe2mv4.restype = None
        L.orc_ebe2mv4.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip, _dp, _dp, _dp,
                                  ctypes.c_int, _dp, _dp]
        L._blk_ready = True
    return L


def block_ops(ndof, nnodes, vert, node_id, neq, A, P, p, F):
    """Every multi-dof EBE operator of the oracle on one input set."""
    L = _blk_lib()
    vert = _c(vert, np.int32).reshape(-1)
    node_id = _c(node_id, np.int32).reshape(-1)
    nel = vert.size // 3
    m = 3 * ndof
    A = _c(A, np.float64).reshape(-1)
    lm = np.zeros(nel * m, np.int32)
    L.orc_fill_lm_blk(ndof, nel, vert, node_id, neq, lm)
    Q = np.zeros(neq + 1)
    L.orc_ebemv_blk(ndof, neq, nel, lm, A, np.array(P, dtype=np.float64), Q)
    d2 = ndof * ndof
    BD = np.zeros(nnodes * d2)
    invBD = np.zeros(nnodes * d2)
    Fo = np.array(F, dtype=np.float64)
    L.orc_blockdiag_setup(ndof, nnodes, nel, neq, vert, node_id, A, BD, invBD, Fo.ctypes.data)
    Z = np.array(p, dtype=np.float64)
    L.orc_blockdiag_apply(ndof, nnodes, neq, node_id, invBD, np.array(p, dtype=np.float64), Z)
    out = dict(lm=lm.reshape(nel, m), Q=Q, BD=BD.reshape(nnodes, d2), invBD=invBD.reshape(nnodes, d2), F=Fo, Z=Z)
    if ndof == 4:
        for key, inv in (("Q2", 1), ("Q2no", 0)):
            Qx = np.zeros(neq + 1)
            L.orc_ebe2mv4(nnodes, neq, nel, lm, node_id, A, BD, invBD, inv, np.array(P, dtype=np.float64), Qx)
            out[key] = Qx
    return out


def last_times(npicard=0, fast=False):
    """(phase times [setup, build, precond_setup, solve], per-step times) of
    the last run_transport, in seconds."""
    L = lib(fast)
    t = np.zeros(4)
    L.orc_get_times(t)
    s = np.zeros(max(npicard, 1))
    L.orc_get_step_times(s, max(npicard, 1))
    return t, s[:npicard]


def csr_pattern(neq, lm):
    """(IA, JA, sbe) of csr_Initialization for an lm array [nel, 3]."""
    L = lib()
    lm = _c(lm, np.int32).reshape(-1)
    nel = lm.size // 3
    nnz = L.orc_csr_pattern(neq, nel, lm, None, None, None)
    IA = np.zeros(neq + 1, np.int32)
    JA = np.zeros(max(nnz, 1), np.int32)
    sbe = np.zeros(9 * nel, np.int32)
    L.orc_csr_pattern(neq, nel, lm, IA.ctypes.data, JA.ctypes.data, sbe.ctypes.data)
    return IA, JA[:nnz], sbe.reshape(nel, 9)


def fill_lm(node_type, vert):
    L = lib()
    node_type = _c(node_type, np.int32)
    vert = _c(vert, np.int32).reshape(-1)
    node_id = np.zeros(node_type.size, np.int32)
    lm = np.zeros(vert.size, np.int32)
    neq = L.orc_fill_lm(node_type.size, node_type, vert.size // 3, vert, node_id, lm)
    return neq, node_id, lm.reshape(-1, 3)


def symrcm(IA, JA):
    L = lib()
    n = IA.size - 1
    perm = np.zeros(n, np.int32)
    L.orc_symrcm(n, _c(IA, np.int32), _c(JA, np.int32), perm)
    return perm


def csrmv(IA, JA, AA, P):
    L = lib()
    n = IA.size - 1
    Q = np.zeros(n + 1)
    L.orc_csrmv(n, _c(IA, np.int32), _c(JA, np.int32), _c(AA, np.float64), _c(P, np.float64), Q)
    return Q


def ebemv(neq, lm, A, P):
    L = lib()
    Q = np.zeros(neq + 1)
    P = np.array(P, dtype=np.float64, copy=True)
    L.orc_ebemv(neq, len(lm), _c(lm, np.int32).reshape(-1), _c(A, np.float64).reshape(-1), P, Q)
    return Q


def edemv(neq, lm2, A, P):
    L = lib()
    Q = np.zeros(neq + 1)
    P = np.array(P, dtype=np.float64, copy=True)
    L.orc_edemv(neq, len(lm2), _c(lm2, np.int32).reshape(-1), _c(A, np.float64).reshape(-1), P, Q)
    return Q


def ilu0(IA, JA, AA):
    L = lib()
    n = IA.size - 1
    LU = np.zeros(IA[-1] + 1)
    Dinv = np.zeros(n + 1)
    rc = L.orc_ilu0_factor(n, _c(IA, np.int32), _c(JA, np.int32), _c(AA, np.float64), LU, Dinv)
    if rc:
        raise ZeroDivisionError(f"zero pivot in row {rc - 1}")
    return LU, Dinv


def iluk_pattern(IA, JA, p):
    """LEVEL_OF_FILL_lu: the ILU(p) pattern (fIA, fJA), rows lower ascending,
    diagonal, upper in elimination order."""
    L = lib()
    L.orc_iluk_pattern.restype = ctypes.c_int
    L.orc_iluk_pattern.argtypes = [ctypes.c_int, _ip, _ip, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    IA, JA = _c(IA, np.int32), _c(JA, np.int32)
    n = IA.size - 1
    nnz = L.orc_iluk_pattern(n, IA, JA, int(p), None, None)
    fIA = np.zeros(n + 1, np.int32)
    fJA = np.zeros(nnz, np.int32)
    L.orc_iluk_pattern(n, IA, JA, int(p), fIA.ctypes.data, fJA.ctypes.data)
    return fIA, fJA


def iluk(IA, JA, AA, p):
    """ILUp (ILUp_precond_setup.c:66-167) with level of fill p: (fIA, fJA, LU,
    Dinv) on the filled pattern."""
    fIA, fJA = iluk_pattern(IA, JA, p)
    L = lib()
    L.orc_iluk_scatter.restype = None
    L.orc_iluk_scatter.argtypes = [ctypes.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
    n = IA.size - 1
    fA = np.zeros(fJA.size + 1)
    L.orc_iluk_scatter(n, _c(IA, np.int32), _c(JA, np.int32), _c(AA, np.float64), fIA, fJA, fA)
    LU, Dinv = ilu0(fIA, fJA, fA)
    return fIA, fJA, LU, Dinv


def ilu0_apply(IA, JA, LU, Dinv, p):
    L = lib()
    n = IA.size - 1
    z = np.zeros(n + 1)
    L.orc_ilu0_apply(n, _c(IA, np.int32), _c(JA, np.int32), _c(LU, np.float64),
                     _c(Dinv, np.float64), _c(p, np.float64), z)
    return z


def csr_gmres(IA, JA, AA, B, use_ilu0=True, kmax=30, lmax=1000, tol=1e-8):
    """pgmres on an assembled CSR system; returns (X, iterations, M^-1 B)."""
    L = lib()
    n = IA.size - 1
    B = np.array(B, dtype=np.float64, copy=True)
    X = np.zeros(n + 1)
    it = L.orc_csr_gmres(n, _c(IA, np.int32), _c(JA, np.int32), _c(AA, np.float64),
                         1 if use_ilu0 else 0, kmax, lmax, tol, B, X)
    return X, it, B


def _amg_pack(levels):
    n = np.array([lv[0].size - 1 for lv in levels], np.int32)
    IA = np.concatenate([lv[0] for lv in levels]).astype(np.int32)
    JA = np.concatenate([lv[1] for lv in levels]).astype(np.int32)
    AA = np.concatenate([lv[2] for lv in levels]).astype(np.float64)
    rm = np.concatenate([lv[3] for lv in levels[:-1]] + [np.zeros(1, np.int32)]).astype(np.int32)
    return n, IA, JA, AA, rm


def amg_vcycle(levels, omega, nr, q):
    """One dpa_Vcycle_precond over levels [(IA, JA, AA, rmatch), ...]."""
    n, IA, JA, AA, rm = _amg_pack(levels)
    z = np.zeros(n[0])
    lib().orc_amg_vcycle(len(levels), n, IA, JA, AA, rm, float(omega), int(nr), _c(q[: n[0]], np.float64), z)
    return z


def amg_gmres(levels, omega, nr, B, kmax=30, lmax=1000, tol=1e-8):
    """pgmres + AMG V-cycle on the level-0 system; returns (X, iterations, M^-1 B)."""
    n, IA, JA, AA, rm = _amg_pack(levels)
    B = np.array(B[: n[0]], dtype=np.float64, copy=True)
    B = np.concatenate([B, [0.0]])
    X = np.zeros(n[0] + 1)
    it = lib().orc_amg_gmres(len(levels), n, IA, JA, AA, rm, float(omega), int(nr), kmax, lmax, tol, B, X)
    return X[: n[0]], it, B[: n[0]]


class EulerParams(ctypes.Structure):
    """orc_euler of oracle.h."""
    _fields_ = [("nnodes", ctypes.c_int), ("nel", ctypes.c_int), ("neq", ctypes.c_int),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("vert", ctypes.c_void_p),
                ("node_id", ctypes.c_void_p), ("upresc", ctypes.c_void_p),
                ("gamma", ctypes.c_double), ("mach", ctypes.c_double), ("dimensionless", ctypes.c_int),
                ("alpha", ctypes.c_double), ("dt", ctypes.c_double), ("stab_tol", ctypes.c_double)]


def _euler(x, y, vert, node_id, neq, upresc, gamma, alpha, dt, stab_tol, mach=1.0, dimensionless=False):
    keep = [_c(x, np.float64), _c(y, np.float64), _c(vert, np.int32).reshape(-1),
            _c(node_id, np.int32).reshape(-1), _c(upresc, np.float64).reshape(-1)]
    p = EulerParams(len(keep[0]), len(keep[2]) // 3, int(neq), *(k.ctypes.data for k in keep),
                    float(gamma), float(mach), int(bool(dimensionless)), float(alpha), float(dt),
                    float(stab_tol))
    return p, keep


def euler_build(x, y, vert, node_id, neq, upresc, u, du, gamma=1.4, alpha=0.5, dt=1e-3,
                stab_tol=1e-6, mach=1.0, dimensionless=False):
    """Build_M_K_F_SUPG: (Ae [nel,144], R [neq+1])."""
    L = lib()
    p, keep = _euler(x, y, vert, node_id, neq, upresc, gamma, alpha, dt, stab_tol, mach, dimensionless)
    Ae = np.zeros((p.nel, 144))
    R = np.zeros(neq + 1)
    L.orc_euler_build.restype = None
    L.orc_euler_build.argtypes = [ctypes.POINTER(EulerParams), _dp, _dp, _dp, _dp]
    L.orc_euler_build(ctypes.byref(p), _c(u, np.float64), _c(du, np.float64), Ae, R)
    return Ae, R


def euler_predictor(x, y, vert, node_id, neq, upresc, u0, nsteps, ncorr=2, gamma=1.4, alpha=0.5,
                    dt=1e-3, stab_tol=1e-6, kmax=30, lmax=100, tol=1e-8, mach=1.0, dimensionless=False,
                    fast=False):
    """Predictor_Old with StopByIterations: (u after each step [nsteps, neq+1],
    GMRES iterations [nsteps, ncorr]); fast: the -Ofast build (timing)."""
    L = lib(fast)
    p, keep = _euler(x, y, vert, node_id, neq, upresc, gamma, alpha, dt, stab_tol, mach, dimensionless)
    u = np.array(u0, dtype=np.float64)
    uhist = np.zeros((nsteps, neq + 1))
    iters = np.zeros((nsteps, ncorr), np.int32)
    L.orc_euler_predictor.restype = ctypes.c_int
    L.orc_euler_predictor.argtypes = [ctypes.POINTER(EulerParams), ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp, _ip]
    L.orc_euler_predictor(ctypes.byref(p), kmax, lmax, tol, nsteps, ncorr, u, uhist, iters)
    return uhist, iters


class NSParams(ctypes.Structure):
    """orc_ns of oracle.h."""
    _fields_ = [("nnodes", ctypes.c_int), ("nel", ctypes.c_int), ("neq", ctypes.c_int),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("vert", ctypes.c_void_p),
                ("node_id", ctypes.c_void_p), ("upresc", ctypes.c_void_p), ("f", ctypes.c_void_p),
                ("re", ctypes.c_double), ("velmax", ctypes.c_double)]


def _ns(x, y, vert, node_id, neq, upresc, f, re, velmax):
    keep = [_c(x, np.float64), _c(y, np.float64), _c(vert, np.int32).reshape(-1),
            _c(node_id, np.int32).reshape(-1), _c(upresc, np.float64).reshape(-1),
            _c(f, np.float64).reshape(-1)]
    p = NSParams(len(keep[0]), len(keep[2]) // 3, int(neq), *(k.ctypes.data for k in keep), float(re),
                 float(velmax))
    return p, keep


def ns_builds(x, y, vert, node_id, neq, upresc, f, re, velmax, us):
    """Consecutive Build_K_F_MS calls on the states us (first call flagged as
    the run's first): (Ae [nb, nel, 81], F [nb, neq+1], delta_old, normres_old)."""
    L = lib()
    p, keep = _ns(x, y, vert, node_id, neq, upresc, f, re, velmax)
    L.orc_ns_build.restype = None
    L.orc_ns_build.argtypes = [ctypes.POINTER(NSParams), _dp, ctypes.c_int, _dp, _dp, _dp, _dp]
    dold = np.zeros(p.nel)
    nold = np.zeros(p.nel)
    Ae = np.zeros((len(us), p.nel, 81))
    F = np.zeros((len(us), neq + 1))
    for b, u in enumerate(us):
        A1 = np.zeros(p.nel * 81)
        F1 = np.zeros(neq + 1)
        L.orc_ns_build(ctypes.byref(p), _c(u, np.float64), 1 if b == 0 else 0, dold, nold, A1, F1)
        Ae[b] = A1.reshape(p.nel, 81)
        F[b] = F1
    return Ae, F, dold, nold


def ns_newton(x, y, vert, node_id, neq, upresc, f, re, velmax, kmax=30, lmax=50, eta0=0.1, ecase=2,
              tolnl=1e-6, maxit=10):
    """Process.c's damped Newton: (uhist [n, neq+1], |F| [n], w [n], GMRES iterations [n])."""
    L = lib()
    p, keep = _ns(x, y, vert, node_id, neq, upresc, f, re, velmax)
    L.orc_ns_newton.restype = ctypes.c_int
    L.orc_ns_newton.argtypes = [ctypes.POINTER(NSParams), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _ip]
    uh = np.zeros((maxit, neq + 1))
    nF = np.zeros(maxit)
    w = np.zeros(maxit)
    g = np.zeros(maxit, np.int32)
    n = L.orc_ns_newton(ctypes.byref(p), kmax, lmax, eta0, ecase, tolnl, maxit, uh, nF, w, g)
    return uh[:n], nF[:n], w[:n], g[:n]
