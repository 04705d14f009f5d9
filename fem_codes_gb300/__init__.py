"""fem_codes_gb300 -- GB300-native steady 2D stabilised-FEM solve loop.

Python access to libfemgpu.so (C ABI, include/femgpu.h).  The class
:class:`SSTransport` mirrors the reference's steady-transport driver
(01_SS_Transport_Equation/2D/01_CommonFiles): ``Preprocess`` is the
constructor, and ``Build``, ``precond_setup``, ``precond``,
``ProductMatrixVector``, ``solver`` and ``Process`` carry the names of the
function pointers they replace (SSTranspEquation.h:97-121), with the same
argument meaning: vectors of length neq+1, slot neq the dump of prescribed
dofs.  There is no CPU fallback: every call runs the CUDA kernels, and a
missing library or GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB, build as _build

__all__ = ["SSTransport", "Euler", "NavierStokes", "AMG", "FemGpuError", "load", "OPTS"]

_lib = None

ERRORS = {
    -1: "bad argument", -2: "CUDA error", -3: "device allocation failed",
    -4: "zero pivot", -5: "not converged", -6: "GMRES breakdown", -7: "device wait timeout",
    -8: "mesh/structure unsupported", -9: "call order",
}

# Parameter-deck strings (Preprocess.c:44-62) -> ABI enums.
OPTS = {
    "scheme": {"EBE": 0, "EDE": 1, "CSR": 2},
    "reorder": {"NOT": 0, "SYMRCM": 1},
    "precond": {"NOT": 0, "ILU0": 1, "DIAG": 2, "BLOCKDIAG": 3, "LEARNED": 4, "AMG": 5},
    "shock": {"CAU": 0, "YZBETA": 1, "CAUDD": 2},
    "hshock": {"2SQRTAREA": 0, "SQRTAREA": 1, "OPTION1": 2, "OPTION2": 3},
    "precision": {"FP64": 0, "MIXED": 1, "MIXED_IR": 2},
    "solver": {"GMRES": 0, "PGMRES": 0, "FGMRES": 1},
}


def _precond_code(precond):
    """femgpu_precond of a deck-style preconditioner name and its level of
    fill: "ILU<p>" (ILUp_precond_setup.c:15) -> (FEMGPU_PREC_ILU0, p)."""
    name = precond.upper()
    if name.startswith("ILU") and name[3:].isdigit():
        return OPTS["precond"]["ILU0"], int(name[3:])
    return OPTS["precond"][name], 0


class FemGpuError(RuntimeError):
    def __init__(self, code, where=""):
        msg = ERRORS.get(code, f"error {code}")
        detail = _lib.femgpu_last_error().decode() if _lib is not None else ""
        super().__init__(f"{where}: {msg} ({code}) {detail}".strip())
        self.code = code


class TransientOpts(ctypes.Structure):
    _fields_ = [("stab", ctypes.c_int), ("alpha", ctypes.c_double), ("dt", ctypes.c_double),
                ("final_time", ctypes.c_double), ("stop_norm", ctypes.c_int), ("max_corr", ctypes.c_int),
                ("nonlin_tol", ctypes.c_double), ("steady_stop", ctypes.c_int), ("time_tol", ctypes.c_double),
                ("method", ctypes.c_int)]


class Opts(ctypes.Structure):
    _fields_ = [("scheme", ctypes.c_int), ("reorder", ctypes.c_int), ("precond", ctypes.c_int),
                ("shock", ctypes.c_int), ("hshock", ctypes.c_int), ("outflow", ctypes.c_int),
                ("kmax", ctypes.c_int), ("lmax", ctypes.c_int), ("tol", ctypes.c_double),
                ("nonlin_tol", ctypes.c_double), ("precision", ctypes.c_int), ("ir_max", ctypes.c_int),
                ("solver", ctypes.c_int), ("inner_tol", ctypes.c_double), ("stall_ratio", ctypes.c_double),
                ("ilu_blocks", ctypes.c_int), ("ilu_level", ctypes.c_int)]


class EulerOpts(ctypes.Structure):
    """femgpu_euler_opts of femgpu.h."""
    _fields_ = [("gamma", ctypes.c_double), ("mach", ctypes.c_double), ("dimensionless", ctypes.c_int),
                ("alpha", ctypes.c_double), ("dt", ctypes.c_double), ("stab_tol", ctypes.c_double),
                ("precond", ctypes.c_int), ("solver", ctypes.c_int), ("kmax", ctypes.c_int),
                ("lmax", ctypes.c_int), ("tol", ctypes.c_double), ("ncorr", ctypes.c_int),
                ("precision", ctypes.c_int), ("scheme", ctypes.c_int), ("ilu_blocks", ctypes.c_int),
                ("scaling", ctypes.c_int), ("shock", ctypes.c_int), ("invY", ctypes.c_double * 4),
                ("stab", ctypes.c_int), ("method", ctypes.c_int)]


class NSOpts(ctypes.Structure):
    """femgpu_ns_opts of femgpu.h."""
    _fields_ = [("re", ctypes.c_double), ("velmax", ctypes.c_double), ("precond", ctypes.c_int),
                ("solver", ctypes.c_int), ("kmax", ctypes.c_int), ("lmax", ctypes.c_int),
                ("eta0", ctypes.c_double), ("eta_case", ctypes.c_int), ("tol_nl", ctypes.c_double),
                ("scheme", ctypes.c_int), ("ilu_blocks", ctypes.c_int)]


class Deck(ctypes.Structure):
    """femgpu_deck of femgpu.h (a parameter deck as the drivers read it)."""
    _fields_ = [("equation", ctypes.c_int)] + \
        [(n, ctypes.c_char * k) for n, k in (
            ("Experiments", 200), ("ProblemTitle", 300), ("Solver", 200), ("Preconditioner", 1000),
            ("Scaling", 200), ("reordering", 200), ("MatrixVectorProductScheme", 200), ("StabilizationForm", 200),
            ("ShockCapture", 200), ("h_Shock", 200), ("OutputFlow", 200), ("TimeIntegration", 200),
            ("StopAtSteadyState", 200), ("Dimensionless", 200), ("StopMulticorrection", 200))] + \
        [(n, ctypes.c_double) for n in ("SolverTolerance", "NonLinearTolerance", "TimeIntegrationTolerance",
                                       "StabilizationTolerance", "Alpha", "DeltaT", "FinalTime", "Mach")] + \
        [("invY", ctypes.c_double * 4)] + \
        [(n, ctypes.c_double) for n in ("ReynoldsNumber", "VelMax", "SolverToleranceNonLin")] + \
        [(n, ctypes.c_int) for n in ("SolverMaxIter", "KrylovBasisVectorsQuantity", "LinearMaxIter",
                                    "NonLinearMaxIter", "SolverToleranceCase", "nnodes", "nel")]

    def as_dict(self):
        out = {}
        for name, typ in self._fields_:
            v = getattr(self, name)
            if isinstance(v, bytes):
                v = v.decode()
            elif name == "invY":
                v = list(v)
            out[name] = v
        return out


_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)


def load(build_if_needed: bool = True) -> ctypes.CDLL:
    """Load libfemgpu.so (building it first if sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build()
    if not os.path.exists(LIB):
        raise FemGpuError(-2, f"libfemgpu.so missing at {LIB}")
    L = ctypes.CDLL(LIB)
    L.femgpu_last_error.restype = ctypes.c_char_p
    L.femgpu_transport_default_opts.argtypes = [ctypes.POINTER(Opts)]
    L.femgpu_transport_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(Opts), ctypes.c_int,
                                          _vp, _vp, _vp, ctypes.c_int, _vp, ctypes.c_double,
                                          ctypes.c_double, _vp, _vp, _vp, _vp]
    L.femgpu_transport_destroy.argtypes = [_vp]
    L.femgpu_transport_destroy.restype = None
    for name, args in {
        "femgpu_transport_set_stream": [_vp, _vp],
        "femgpu_transport_info": [_vp, _vp],
        "femgpu_transport_ilu_blocks": [_vp, _vp, ctypes.c_int],
        "femgpu_transport_ilu_chain": [_vp, _vp],
        "femgpu_ilu_block_cut": [ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, ctypes.c_int],
        "femgpu_iluk_pattern": [ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int],
        "femgpu_deck_read": [ctypes.c_char_p, ctypes.c_int, _vp],
        "femgpu_deck_mesh_file": [_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int],
        "femgpu_mesh_read": [ctypes.c_char_p, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_mesh_side_types": [ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp],
        "femgpu_transport_set_sweep_wait": [_vp, ctypes.c_int],
        "femgpu_euler_set_slip": [_vp, _vp, _vp, _vp],
        "femgpu_euler_scale": [_vp, _vp, _vp],
        "femgpu_transport_set_transient": [_vp, _vp],
        "femgpu_transport_set_bubbles": [_vp, _vp, _vp],
        "femgpu_transport_operator_dev": [_vp, _vp, _vp],
        "femgpu_transport_build_transient": [_vp, _vp, _vp, _vp, _vp],
        "femgpu_transport_predictor": [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_int],
        "femgpu_deck_transport_opts": [_vp, _vp],
        "femgpu_deck_euler_opts": [_vp, _vp],
        "femgpu_deck_transient_opts": [_vp, _vp, _vp],
        "femgpu_euler_set_build_params": [_vp, ctypes.c_double, ctypes.c_double],
        "femgpu_euler_set_bubbles": [_vp, _vp],
        "femgpu_euler_state": [_vp, _vp, _vp],
        "femgpu_deck_ns_opts": [_vp, _vp],
        "femgpu_deck_amg": [_vp, _vp, _vp, _vp, _vp],
        "femgpu_ilu_chain_segments": [ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp,
                                      ctypes.c_int, ctypes.c_int],
        "femgpu_transport_get_pattern": [_vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_transport_build": [_vp, _vp, _vp, _vp],
        "femgpu_transport_precond_setup": [_vp, ctypes.c_int, _vp],
        "femgpu_transport_precond": [_vp, _vp, _vp],
        "femgpu_transport_matvec": [_vp, _vp, _vp],
        "femgpu_transport_solve": [_vp, _vp, _ip],
        "femgpu_transport_solve_bx": [_vp, _vp, _vp, _ip],
        "femgpu_transport_process": [_vp, ctypes.c_int, _vp, _vp],
        "femgpu_transport_build_dev": [_vp],
        "femgpu_transport_precond_setup_dev": [_vp, ctypes.c_int],
        "femgpu_transport_matvec_dev": [_vp, _vp, _vp],
        "femgpu_transport_precond_dev": [_vp, _vp, _vp],
        "femgpu_transport_solve_dev": [_vp, _ip],
        "femgpu_transport_true_residual": [_vp, ctypes.POINTER(ctypes.c_double)],
        "femgpu_transport_last_times": [_vp, _vp],
        "femgpu_transport_write_vtu": [_vp, ctypes.c_char_p, _vp],
        "femgpu_csrmv_f64": [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_csrmv_f64_fused": [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_csrmv_f32": [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp],
    }.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.femgpu_euler_default_opts.argtypes = [ctypes.POINTER(EulerOpts)]
    L.femgpu_euler_default_opts.restype = None
    L.femgpu_euler_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(EulerOpts), ctypes.c_int, _vp, _vp,
                                      ctypes.c_int, _vp, _vp, ctypes.c_int, _vp]
    L.femgpu_euler_create.restype = ctypes.c_int
    L.femgpu_euler_destroy.argtypes = [_vp]
    L.femgpu_euler_destroy.restype = None
    for name, args in {
        "femgpu_euler_set_stream": [_vp, _vp],
        "femgpu_euler_build": [_vp, _vp, _vp, _vp, _vp],
        "femgpu_euler_build_dev": [_vp],
        "femgpu_euler_precond_setup": [_vp, _vp],
        "femgpu_euler_precond_setup_dev": [_vp],
        "femgpu_euler_solve": [_vp, _vp, _vp, _ip],
        "femgpu_euler_csr": [_vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_euler_set_amg": [_vp, _vp],
        "femgpu_euler_solve_dev": [_vp, _ip],
        "femgpu_euler_predictor": [_vp, _vp, ctypes.c_int, _vp, _vp],
        "femgpu_euler_predictor_dev": [_vp, ctypes.c_int, _vp],
        "femgpu_euler_last_times": [_vp, _vp],
    }.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.femgpu_ns_default_opts.argtypes = [ctypes.POINTER(NSOpts)]
    L.femgpu_ns_default_opts.restype = None
    L.femgpu_ns_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(NSOpts), ctypes.c_int, _vp, _vp,
                                   ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp]
    L.femgpu_ns_create.restype = ctypes.c_int
    L.femgpu_ns_destroy.argtypes = [_vp]
    L.femgpu_ns_destroy.restype = None
    for name, args in {
        "femgpu_ns_set_stream": [_vp, _vp],
        "femgpu_ns_reset": [_vp],
        "femgpu_ns_build": [_vp, _vp, _vp, _vp],
        "femgpu_ns_build_dev": [_vp],
        "femgpu_ns_precond_setup": [_vp, _vp],
        "femgpu_ns_solve": [_vp, _vp, _vp, _ip],
        "femgpu_ns_set_tol": [_vp, ctypes.c_double],
        "femgpu_ns_set_amg": [_vp, _vp],
        "femgpu_ns_newton": [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp],
        "femgpu_ns_csr": [_vp, _vp, _vp, _vp, _vp],
    }.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    for name in ("femgpu_ns_u_dev", "femgpu_ns_ebe"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = _vp
    L.femgpu_gnn_nparams.restype = ctypes.c_int
    L.femgpu_gnn_nparams.argtypes = []
    L.femgpu_gnn_destroy.argtypes = [_vp]
    L.femgpu_gnn_destroy.restype = None
    L.femgpu_amg_destroy.argtypes = [_vp]
    L.femgpu_amg_destroy.restype = None
    for name, args in {
        "femgpu_gnn_create": [ctypes.POINTER(_vp), ctypes.c_int, _vp],
        "femgpu_gnn_set_stream": [_vp, _vp],
        "femgpu_gnn_set_params": [_vp, _vp],
        "femgpu_gnn_get_params": [_vp, _vp],
        "femgpu_gnn_get_grad": [_vp, _vp],
        "femgpu_gnn_attach_csr": [_vp, ctypes.c_int, _vp, _vp, _vp],
        "femgpu_gnn_attach_csr_dev": [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp],
        "femgpu_gnn_apply": [_vp, _vp, _vp],
        "femgpu_gnn_apply_dev": [_vp, _vp, _vp],
        "femgpu_gnn_loss_grad_dev": [_vp, _vp, _vp, _vp, ctypes.c_int, _vp],
        "femgpu_gnn_loss_grad": [_vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_gnn_adam_step": [_vp, ctypes.c_float, ctypes.c_float],
        "femgpu_gnn_set_loss": [_vp, ctypes.c_int],
        "femgpu_transport_set_learned": [_vp, _vp],
        "femgpu_amg_create": [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int],
        "femgpu_amg_set_stream": [_vp, _vp],
        "femgpu_amg_setup": [_vp, ctypes.c_int, _vp, _vp, _vp],
        "femgpu_amg_levels": [_vp],
        "femgpu_amg_level": [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp],
        "femgpu_amg_apply": [_vp, _vp, _vp],
        "femgpu_amg_apply_dev": [_vp, _vp, _vp],
        "femgpu_transport_set_amg": [_vp, _vp],
        "femgpu_dpa_match": [ctypes.c_int, _vp, _vp, _vp, ctypes.c_double, _vp],
        "femgpu_dpa_galerkin": [ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "femgpu_transport_krylov_pairs": [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int],
        "femgpu_transport_csr_dev": [_vp, _vp, _vp, _vp],
    }.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    for name in ("femgpu_euler_u_dev", "femgpu_euler_ebe"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = _vp
    for name in ("femgpu_transport_u_dev", "femgpu_transport_F_dev"):
        getattr(L, name).argtypes = [_vp]
        getattr(L, name).restype = _vp
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def ilu_block_cut(IA, JA, P):
    """First row of each block ILU(0) run (plus the row count) for a CSR
    pattern with ascending columns, computed on the host exactly as a
    transport context with ilu_blocks = P cuts its own (needs no GPU)."""
    L = load()
    IA = np.ascontiguousarray(IA, dtype=np.int32)
    JA = np.ascontiguousarray(JA, dtype=np.int32)
    n = IA.size - 1
    first = np.zeros(max(min(P, n), 1) + 1, np.int32)
    rc = L.femgpu_ilu_block_cut(n, _ptr(IA), _ptr(JA), int(P), _ptr(first), first.size)
    if rc < 0:
        raise FemGpuError(rc, "ilu_block_cut")
    return first[: rc + 1]


EQUATIONS = {"transport": 0, "euler": 1, "ns": 2, "transient": 3}
NODE_TYPES = {"transport": 1, "euler": 4, "ns": 3, "transient": 1}
MESH_NO_ELEM_TYPE = 0x100            # FEMGPU_MESH_NO_ELEM_TYPE: the transient driver's element lines


def read_deck(path, equation="transport"):
    """A parameter deck as the driver's Preprocess reads it (femgpu_deck):
    the Deck structure (``as_dict()`` for a dict)."""
    L = load()
    d = Deck()
    rc = L.femgpu_deck_read(os.fsencode(path), EQUATIONS[equation], ctypes.byref(d))
    if rc:
        raise FemGpuError(rc, f"read_deck {path}")
    return d


def deck_mesh_file(deck, directory):
    """The mesh file a driver opens for a deck: <dir>/<title>_<nnodes>_<nel>.dat."""
    L = load()
    buf = ctypes.create_string_buffer(4096)
    rc = L.femgpu_deck_mesh_file(ctypes.byref(deck), os.fsencode(directory), buf, 4096)
    if rc:
        raise FemGpuError(rc, "deck_mesh_file")
    return buf.value.decode()


def read_mesh(path, equation="transport"):
    """A mesh file in the drivers' format: dict(x, y, node_type [nnodes, k],
    vert [nel, 3], elem_type).  For transport the element types are the
    boundary sides its Preprocess sets (femgpu_mesh_side_types); Euler and
    Navier-Stokes keep the file's column; the transient transport files have
    none (element types 0)."""
    L = load()
    k = NODE_TYPES[equation]
    kf = k | (MESH_NO_ELEM_TYPE if equation == "transient" else 0)
    nn, ne = ctypes.c_int(0), ctypes.c_int(0)
    p = os.fsencode(path)
    rc = L.femgpu_mesh_read(p, kf, ctypes.byref(nn), ctypes.byref(ne), None, None, None, None, None)
    if rc:
        raise FemGpuError(rc, f"read_mesh {path}")
    x, y = np.zeros(nn.value), np.zeros(nn.value)
    nt = np.zeros((nn.value, k), np.int32)
    vert = np.zeros((ne.value, 3), np.int32)
    et = np.zeros(ne.value, np.int32)
    rc = L.femgpu_mesh_read(p, kf, ctypes.byref(nn), ctypes.byref(ne), _ptr(x), _ptr(y), _ptr(nt), _ptr(vert),
                            _ptr(et))
    if rc:
        raise FemGpuError(rc, f"read_mesh {path}")
    if equation == "transport":
        rc = L.femgpu_mesh_side_types(nn.value, _ptr(x), _ptr(y), ne.value, _ptr(vert), _ptr(et))
        if rc:
            raise FemGpuError(rc, f"read_mesh {path}")
    return dict(x=x, y=y, node_type=nt if k > 1 else nt[:, 0].copy(), vert=vert, elem_type=et)


def deck_opts(deck):
    """The deck's strings as the library's options (Opts, EulerOpts or NSOpts;
    for a transient transport deck the pair (Opts, TransientOpts))."""
    L = load()
    eq = deck.equation
    if eq == EQUATIONS["transient"]:
        o, tr = Opts(), TransientOpts()
        rc = L.femgpu_deck_transient_opts(ctypes.byref(deck), ctypes.byref(o), ctypes.byref(tr))
        if rc:
            raise FemGpuError(rc, "deck_opts")
        return o, tr
    o = (Opts, EulerOpts, NSOpts)[eq]()
    f = (L.femgpu_deck_transport_opts, L.femgpu_deck_euler_opts, L.femgpu_deck_ns_opts)[eq]
    rc = f(ctypes.byref(deck), ctypes.byref(o))
    if rc:
        raise FemGpuError(rc, "deck_opts")
    return o


def iluk_pattern(IA, JA, p):
    """The ILU(p) pattern of a CSR pattern (LEVEL_OF_FILL_lu): (fIA, fJA),
    rows stored lower ascending, diagonal, upper in elimination order."""
    L = load()
    IA = np.ascontiguousarray(IA, dtype=np.int32)
    JA = np.ascontiguousarray(JA, dtype=np.int32)
    n = IA.size - 1
    nnz = L.femgpu_iluk_pattern(n, _ptr(IA), _ptr(JA), int(p), None, None, 0)
    if nnz < 0:
        raise FemGpuError(nnz, "iluk_pattern")
    fIA = np.zeros(n + 1, np.int32)
    fJA = np.zeros(nnz, np.int32)
    rc = L.femgpu_iluk_pattern(n, _ptr(IA), _ptr(JA), int(p), _ptr(fIA), _ptr(fJA), nnz)
    if rc < 0:
        raise FemGpuError(rc, "iluk_pattern")
    return fIA, fJA


def ilu_chain_segments(IA, JA, P, lower=True):
    """The chain-scan segmentation of one ILU(0) sweep of a CSR pattern (the
    programs a transport context with ilu_blocks = P builds for its FGMRES and
    FP32 sweeps), computed on the host: dict with slot_row, slot_pred, lstart
    and the level counts."""
    L = load()
    IA = np.ascontiguousarray(IA, dtype=np.int32)
    JA = np.ascontiguousarray(JA, dtype=np.int32)
    n = IA.size - 1
    info = np.zeros(4, np.int32)
    ns = L.femgpu_ilu_chain_segments(n, _ptr(IA), _ptr(JA), int(P), int(lower), _ptr(info), None, None, None, 0, 0)
    if ns < 0:
        raise FemGpuError(ns, "ilu_chain_segments")
    row = np.zeros(ns, np.int32)
    pred = np.zeros(ns, np.int32)
    lstart = np.zeros(int(info[0]) + 1, np.int32)
    rc = L.femgpu_ilu_chain_segments(n, _ptr(IA), _ptr(JA), int(P), int(lower), _ptr(info), _ptr(row), _ptr(pred),
                                     _ptr(lstart), ns, lstart.size)
    if rc < 0:
        raise FemGpuError(rc, "ilu_chain_segments")
    return dict(slot_row=row, slot_pred=pred, lstart=lstart, levels=int(info[0]), deepest=int(info[1]),
                deepest_rows=int(info[2]), width=int(info[3]))


class SSTransport:
    """Steady scalar transport on one GPU (the reference's Preprocess ->
    Process -> pgmres path), built from arrays instead of a mesh file."""

    def __init__(self, x, y, node_type, vert, k, gamma, upresc, beta=None, const_beta=None,
                 fsrc=None, scheme="CSR", reorder="NOT", precond="ILU0", shock="CAU",
                 hshock="2sqrtArea", outflow=False, kmax=30, lmax=1000, tol=1e-8,
                 nonlin_tol=0.0, precision="FP64", ir_max=30, solver="GMRES", inner_tol=1e-4,
                 stall_ratio=0.9, ilu_blocks=0):
        L = load()
        o = Opts()
        L.femgpu_transport_default_opts(ctypes.byref(o))
        o.scheme = OPTS["scheme"][scheme.upper()]
        o.reorder = OPTS["reorder"][reorder.upper()]
        o.precond, o.ilu_level = _precond_code(precond)
        o.shock = OPTS["shock"][shock.upper()]
        o.hshock = OPTS["hshock"][hshock.upper()]
        o.outflow = 1 if outflow else 0
        o.kmax, o.lmax, o.tol, o.nonlin_tol = kmax, lmax, tol, nonlin_tol
        o.precision = OPTS["precision"][precision.upper()]
        o.ir_max = ir_max
        o.solver = OPTS["solver"][solver.upper()]
        o.inner_tol = inner_tol
        o.stall_ratio = stall_ratio
        o.ilu_blocks = int(ilu_blocks)
        self.opts = o
        self._keep = [_f64(x), _f64(y), _i32(node_type), _i32(np.asarray(vert).reshape(-1)),
                      _f64(upresc)]
        self.nnodes = len(x)
        self.nel = self._keep[3].size // 3
        b = None if beta is None else _f64(np.asarray(beta).reshape(-1))
        cb = None if const_beta is None else _f64(const_beta)
        f = None if fsrc is None else _f64(np.asarray(fsrc).reshape(-1))
        self._keep += [b, cb, f]
        h = _vp()
        rc = L.femgpu_transport_create(ctypes.byref(h), ctypes.byref(o), self.nnodes,
                                       _ptr(self._keep[0]), _ptr(self._keep[1]), _ptr(self._keep[2]),
                                       self.nel, _ptr(self._keep[3]), float(k), float(gamma),
                                       _ptr(b), _ptr(cb), _ptr(f), _ptr(self._keep[4]))
        if rc:
            raise FemGpuError(rc, "Preprocess")
        self._h = h
        self._L = L
        info = np.zeros(7, np.int32)
        self._check(L.femgpu_transport_info(h, _ptr(info)), "info")
        self.neq, self.nnzero, self.nedge, self.bandwidth, self.ilu_levels_L, self.ilu_levels_U = \
            (int(v) for v in info[:6])
        self.scheme = scheme.upper()

    @classmethod
    def from_problem(cls, mesh, prob, **kw):
        return cls(mesh.x, mesh.y, prob.node_type, mesh.vert, prob.k, prob.gamma, prob.upresc,
                   beta=prob.beta, fsrc=prob.fsrc, **kw)

    # -- helpers -----------------------------------------------------------
    def _check(self, rc, where):
        if rc:
            raise FemGpuError(rc, where)

    def close(self):
        if getattr(self, "_h", None):
            self._L.femgpu_transport_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        self._check(self._L.femgpu_transport_set_stream(self._h, _vp(stream_ptr)), "set_stream")

    # -- structure ---------------------------------------------------------
    def pattern(self):
        """Device-built storage structure, as the reference holds it."""
        node_id = np.zeros(self.nnodes, np.int32)
        if self.scheme == "CSR":
            IA = np.zeros(self.neq + 1, np.int32)
            JA = np.zeros(max(self.nnzero, 1), np.int32)
            sbe = np.zeros(9 * self.nel, np.int32)
            self._check(self._L.femgpu_transport_get_pattern(self._h, _ptr(IA), _ptr(JA), _ptr(sbe),
                                                             None, _ptr(node_id)), "pattern")
            return dict(IA=IA, JA=JA[: self.nnzero], sbe=sbe.reshape(-1, 9), node_id=node_id)
        if self.scheme == "EDE":
            lm2 = np.zeros(2 * max(self.nedge, 1), np.int32)
            sbe = np.zeros(3 * self.nel, np.int32)
            order = np.zeros(3 * self.nel, np.int32)
            self._check(self._L.femgpu_transport_get_pattern(self._h, None, _ptr(lm2), _ptr(sbe),
                                                             _ptr(order), _ptr(node_id)), "pattern")
            return dict(lm2=lm2[: 2 * self.nedge].reshape(-1, 2), sbe=sbe.reshape(-1, 3),
                        order=order.reshape(-1, 3), node_id=node_id)
        self._check(self._L.femgpu_transport_get_pattern(self._h, None, None, None, None,
                                                         _ptr(node_id)), "pattern")
        return dict(node_id=node_id)

    def storage_len(self):
        if self.scheme == "CSR":
            return self.nnzero + 1
        if self.scheme == "EDE":
            return 4 * (self.nedge + 1)
        return 9 * self.nel

    # -- the reference's function pointers --------------------------------
    def Build(self, u=None, want_matrix=False):
        """FemOtherFunctions->Build: element loop + assembly. Returns (F, A)."""
        F = np.zeros(self.neq + 1)
        A = np.zeros(self.storage_len()) if want_matrix else None
        uu = None if u is None else _f64(u)
        self._check(self._L.femgpu_transport_build(self._h, _ptr(uu), _ptr(F), _ptr(A)), "Build")
        return F, A

    def precond_setup(self, tag=1):
        """FemFunctions->precond_setup: factor, then F := M^-1 F. Returns F."""
        F = np.zeros(self.neq + 1)
        self._check(self._L.femgpu_transport_precond_setup(self._h, int(tag), _ptr(F)), "precond_setup")
        return F

    def precond(self, p):
        """FemFunctions->precond: z = M^-1 p (entries 0..neq-1)."""
        p = _f64(p)
        z = p.copy()
        self._check(self._L.femgpu_transport_precond(self._h, _ptr(p), _ptr(z)), "precond")
        return z

    def ProductMatrixVector(self, P, Q=None):
        """FemFunctions->ProductMatrixVector: Q = A P."""
        P = np.array(P, dtype=np.float64, copy=True)
        Q = np.zeros(self.neq + 1) if Q is None else Q
        self._check(self._L.femgpu_transport_matvec(self._h, _ptr(P), _ptr(Q)), "ProductMatrixVector")
        return Q

    def solver(self, raise_on_nonconvergence=True):
        """FemOtherFunctions->solver (pgmres, 4-argument form): B = F, X = u.
        Returns (u, iterations)."""
        X = np.zeros(self.neq + 1)
        it = ctypes.c_int(0)
        rc = self._L.femgpu_transport_solve(self._h, _ptr(X), ctypes.byref(it))
        if rc and (rc != -5 or raise_on_nonconvergence):
            raise FemGpuError(rc, "solver")
        return X, it.value

    def solver_bx(self, B):
        """6-argument pgmres form: X = solve(B). Returns (X, iterations)."""
        B = _f64(B)
        X = np.zeros(self.neq + 1)
        it = ctypes.c_int(0)
        self._check(self._L.femgpu_transport_solve_bx(self._h, _ptr(B), _ptr(X), ctypes.byref(it)),
                    "solver")
        return X, it.value

    def Process(self, npicard):
        """Picard loop of Process.c. Returns (u history [n, neq+1], iterations)."""
        uh = np.zeros((npicard, self.neq + 1))
        its = np.zeros(npicard, np.int32)
        n = self._L.femgpu_transport_process(self._h, int(npicard), _ptr(uh), _ptr(its))
        if n < 0:
            raise FemGpuError(n, "Process")
        return uh[:n], its[:n]

    def ilu_blocks(self):
        """First row of each block ILU(0) run plus the row count (a 2-entry
        array for global ILU(0))."""
        P = self._L.femgpu_transport_ilu_blocks(self._h, None, 0)
        if P < 0:
            raise FemGpuError(P, "ilu_blocks")
        first = np.zeros(P + 1, np.int32)
        rc = self._L.femgpu_transport_ilu_blocks(self._h, _ptr(first), P + 1)
        if rc < 0:
            raise FemGpuError(rc, "ilu_blocks")
        return first

    def true_residual(self):
        r = ctypes.c_double(0.0)
        self._check(self._L.femgpu_transport_true_residual(self._h, ctypes.byref(r)), "true_residual")
        return r.value

    def last_times(self):
        t = np.zeros(3, np.float32)
        self._check(self._L.femgpu_transport_last_times(self._h, _ptr(t)), "last_times")
        return t

    # device-resident path (no host copies)
    def build_dev(self):
        self._check(self._L.femgpu_transport_build_dev(self._h), "build_dev")

    def precond_setup_dev(self, tag=1):
        self._check(self._L.femgpu_transport_precond_setup_dev(self._h, int(tag)), "precond_setup_dev")

    def solve_dev(self, raise_on_nonconvergence=True):
        it = ctypes.c_int(0)
        rc = self._L.femgpu_transport_solve_dev(self._h, ctypes.byref(it))
        if rc and (rc != -5 or raise_on_nonconvergence):
            raise FemGpuError(rc, "solve_dev")
        return it.value

    def write_vtu(self, path, u=None):
        """Paraview_Output: the reference's VTU file of the solution u [neq+1]
        (None: the last solution) at path."""
        uu = None if u is None else _f64(u)
        self._check(self._L.femgpu_transport_write_vtu(self._h, os.fsencode(path), _ptr(uu)), "write_vtu")

    def ilu_chain(self):
        """1 when the ILU(0) sweeps of FGMRES and of the FP32 solves run the
        chain-scan programs, else 0 (femgpu_transport_ilu_chain)."""
        rc = self._L.femgpu_transport_ilu_chain(self._h, None)
        if rc < 0:
            raise FemGpuError(rc, "ilu_chain")
        return rc

    # -- the transient driver (02_Transport_Equation/2D) --------------------
    def set_transient(self, stab="SUPG", alpha=0.5, dt=1e-2, final_time=1.0, stop="ITERATION", max_corr=2,
                      nonlin_tol=1e-3, steady="NOT", time_tol=1e-6, method="Predictor1"):
        """Switch to the transient driver: Build_M_K_R_SUPG / Build_M_K_R_DD
        and the deck's TimeIntegration (Predictor1 | Predictor1_BDF |
        Predictor1_TRBDF2, and with DD Predictor2 | Predictor2_BDF |
        Predictor2_TRBDF2, which build with Build_M_F_DD) with its
        StopMulticorrection (ITERATION | NORM) and StopAtSteadyState
        (YES | NOT)."""
        o = TransientOpts(stab={"SUPG": 0, "DD": 1}[stab.upper()], alpha=alpha, dt=dt, final_time=final_time,
                          stop_norm={"ITERATION": 0, "NORM": 1}[stop.upper()], max_corr=int(max_corr),
                          nonlin_tol=nonlin_tol, steady_stop={"NOT": 0, "YES": 1}[steady.upper()],
                          time_tol=time_tol,
                          method={"PREDICTOR1": 0, "PREDICTOR1_BDF": 1, "PREDICTOR1_TRBDF2": 2,
                                  "PREDICTOR2": 3, "PREDICTOR2_BDF": 4, "PREDICTOR2_TRBDF2": 5}[method.upper()])
        self._stages = 2 if method.upper().endswith("_TRBDF2") else 1
        self._check(self._L.femgpu_transport_set_transient(self._h, ctypes.byref(o)), "set_transient")

    def build_transient(self, u=None, a=None, want_matrix=False):
        """One transient Build on (u, a): returns (R, storage values or None)."""
        R = np.zeros(self.neq + 1)
        A = np.zeros(self.storage_len()) if want_matrix else None
        uu = None if u is None else _f64(u)
        aa = None if a is None else _f64(a)
        self._check(self._L.femgpu_transport_build_transient(self._h, _ptr(uu), _ptr(aa), _ptr(R), _ptr(A)),
                    "build_transient")
        return R, A

    def set_bubbles(self, uB=None, aB=None):
        """The element bubbles (Predictor2) for the next build_transient."""
        self._check(self._L.femgpu_transport_set_bubbles(self._h, _ptr(None if uB is None else _f64(uB)),
                                                         _ptr(None if aB is None else _f64(aB))), "set_bubbles")

    def predictor(self, u0, max_steps, iters_cap=16):
        """The time loop from u0: dict(u [stages, neq+1], t [steps], ncorr
        [stages], iters [stages, iters_cap]) -- a stage is one multicorrection
        loop, two per TRBDF2 step."""
        u0 = _f64(u0)
        S = getattr(self, "_stages", 1)
        uh = np.zeros((S * max_steps, self.neq + 1))
        th = np.zeros(max_steps)
        nc = np.zeros(S * max_steps, np.int32)
        it = np.zeros((S * max_steps, iters_cap), np.int32)
        n = self._L.femgpu_transport_predictor(self._h, _ptr(u0), int(max_steps), _ptr(uh), _ptr(th), _ptr(nc),
                                               _ptr(it), int(iters_cap))
        if n < 0:
            raise FemGpuError(n, "predictor")
        return dict(u=uh[:S * n], t=th[:n], ncorr=nc[:S * n], iters=it[:S * n])

    def set_sweep_wait(self, spins=-1):
        """Bound on a sweep warp's wait for its dependencies (-1: default);
        also clears the context's device error word."""
        self._check(self._L.femgpu_transport_set_sweep_wait(self._h, int(spins)), "set_sweep_wait")

    def fell_back(self):
        """0, or how the last learned-preconditioned solve continued after a
        stall: 1 ILU(0), 2 the attached AMG context."""
        info = np.zeros(7, np.int32)
        self._check(self._L.femgpu_transport_info(self._h, _ptr(info)), "info")
        return int(info[6])

    def u_dev(self):
        return self._L.femgpu_transport_u_dev(self._h)

    def set_learned(self, gnn):
        """Use a :class:`fem_codes_gb300.learned.MeshGNN` as the
        FEMGPU_PREC_LEARNED right preconditioner."""
        self._gnn = gnn
        self._check(self._L.femgpu_transport_set_learned(self._h, gnn.handle), "set_learned")

    def set_amg(self, amg):
        """Use an :class:`AMG` context as the FEMGPU_PREC_AMG preconditioner
        (its hierarchy is rebuilt from the matrix at every precond_setup), or
        as the fallback of the learned preconditioner."""
        self._amg = amg
        self._check(self._L.femgpu_transport_set_amg(self._h, amg.handle), "set_amg")

    def csr_dev(self):
        """(IA, JA, AA) device pointers of the CSR matrix."""
        p = [_vp(), _vp(), _vp()]
        self._check(self._L.femgpu_transport_csr_dev(self._h, *(ctypes.byref(q) for q in p)), "csr_dev")
        return tuple(q.value for q in p)

    def krylov_pairs(self, V_dev, Z_dev, ld, max_pairs):
        """Copy the last FGMRES cycle's (v_i, M^-1 v_i) pairs into device
        arrays; returns the count."""
        n = self._L.femgpu_transport_krylov_pairs(self._h, int(max_pairs), _vp(V_dev), _vp(Z_dev), int(ld))
        if n < 0:
            raise FemGpuError(n, "krylov_pairs")
        return n


class AMG:
    """Double pairwise aggregation AMG preconditioner, parameters as the
    deck string "AMG 2 NCL beta omega nr" (amg_precond.c:26-105): setup
    builds the 2*NCL+1-level hierarchy on the host (AMG_precond_setup),
    apply runs one V-cycle on the GPU (AMG_precond)."""

    def __init__(self, ncl=2, beta=-1.0, omega=1.0, nr=2):
        L = load()
        self._L = L
        h = _vp()
        rc = L.femgpu_amg_create(ctypes.byref(h), int(ncl), float(beta), float(omega), int(nr))
        if rc:
            raise FemGpuError(rc, "amg_create")
        self._h = h
        self.n = 0

    @classmethod
    def from_spec(cls, spec):
        """From the reference's deck string, e.g. "AMG 2 2 -1 1.0 2"."""
        w = spec.split()
        if len(w) < 6 or w[0] != "AMG" or int(w[1]) != 2:
            raise ValueError(f"only the DPA form 'AMG 2 NCL beta omega nr' is provided: {spec!r}")
        return cls(int(w[2]), float(w[3]), float(w[4]), int(w[5]))

    @property
    def handle(self):
        return self._h

    def _check(self, rc, where):
        if rc:
            raise FemGpuError(rc, where)

    def setup(self, IA, JA, AA):
        IA, JA, AA = _i32(IA), _i32(JA), _f64(AA)
        self.n = IA.size - 1
        self._check(self._L.femgpu_amg_setup(self._h, self.n, _ptr(IA), _ptr(JA), _ptr(AA)), "amg_setup")

    def levels(self):
        return self._L.femgpu_amg_levels(self._h)

    def level(self, l):
        """(IA, JA, AA, rmatch or None) of level l."""
        nn = np.zeros(2, np.int32)
        self._check(self._L.femgpu_amg_level(self._h, l, _ptr(nn), None, None, None, None), "amg_level")
        n, nnz = int(nn[0]), int(nn[1])
        IA, JA, AA = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
        rm = np.zeros(n + 1, np.int32) if l < self.levels() - 1 else None
        self._check(self._L.femgpu_amg_level(self._h, l, _ptr(nn), _ptr(IA), _ptr(JA), _ptr(AA), _ptr(rm)),
                    "amg_level")
        return IA, JA, AA, rm

    def apply(self, q):
        q = _f64(q)
        z = np.zeros(self.n)
        self._check(self._L.femgpu_amg_apply(self._h, _ptr(q), _ptr(z)), "amg_apply")
        return z

    def apply_dev(self, q_ptr, z_ptr):
        self._check(self._L.femgpu_amg_apply_dev(self._h, _vp(q_ptr), _vp(z_ptr)), "amg_apply_dev")

    def close(self):
        if getattr(self, "_h", None):
            self._L.femgpu_amg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Euler:
    """2D Euler equations on one GPU: SUPG+CAU element build, block EBE
    storage with the nodal block-diagonal preconditioner, GMRES and the
    predictor-multicorrector (03_Euler_Equations/2D with SUPG, CAU, EBE,
    Predictor1, StopMulticorrection ITERATION).  ``Build``,
    ``precond_setup``, ``solver`` and ``Predictor`` carry the names of the
    functions they replace (EulerEquations.h:136-170, Predictor_Old.c);
    vectors have length neq+1 with slot neq the dump of prescribed dofs."""

    def __init__(self, x, y, vert, node_id, neq, upresc, gamma=1.4, mach=1.0, dimensionless=False,
                 alpha=0.5, dt=1e-3, stab_tol=1e-6, precond="BlockDiag", solver="GMRES", kmax=30,
                 lmax=100, tol=1e-8, ncorr=2, precision="FP64", scheme="EBE", ilu_blocks=0, scaling="NOT",
                 shock="CAU", invY=(1.0, 1.0, 1.0, 1.0), method="Predictor1", stab="SUPG"):
        L = load()
        o = EulerOpts()
        L.femgpu_euler_default_opts(ctypes.byref(o))
        o.shock = {"CAU": 0, "YZBETA": 1, "CAUDD": 2}[shock.upper()]
        o.stab = {"SUPG": 0, "DD": 1}[stab.upper()]
        o.method = {"PREDICTOR1": 0, "PREDICTOR1_BDF": 1, "PREDICTOR1_TRBDF2": 2}[method.upper()]
        for k in range(4):
            o.invY[k] = float(invY[k])
        o.scheme = OPTS["scheme"][scheme.upper()]
        o.ilu_blocks = int(ilu_blocks)
        o.scaling = {"NOT": 0, "BLOCKSCALING": 1}[scaling.upper()]
        o.gamma, o.mach, o.dimensionless = float(gamma), float(mach), int(bool(dimensionless))
        o.alpha, o.dt, o.stab_tol = float(alpha), float(dt), float(stab_tol)
        o.precond = OPTS["precond"][precond.upper()]
        o.solver = OPTS["solver"][solver.upper()]
        o.kmax, o.lmax, o.tol, o.ncorr = int(kmax), int(lmax), float(tol), int(ncorr)
        o.precision = OPTS["precision"][precision.upper()]
        self.opts = o
        self._keep = [_f64(x), _f64(y), _i32(np.asarray(vert).reshape(-1)),
                      _i32(np.asarray(node_id).reshape(-1)), _f64(np.asarray(upresc).reshape(-1))]
        self.nnodes = len(self._keep[0])
        self.nel = self._keep[2].size // 3
        self.neq = int(neq)
        h = _vp()
        rc = L.femgpu_euler_create(ctypes.byref(h), ctypes.byref(o), self.nnodes, _ptr(self._keep[0]),
                                   _ptr(self._keep[1]), self.nel, _ptr(self._keep[2]), _ptr(self._keep[3]),
                                   self.neq, _ptr(self._keep[4]))
        if rc:
            raise FemGpuError(rc, "Preprocess")
        self._h = h
        self._L = L

    @classmethod
    def from_problem(cls, mesh, prob, **kw):
        return cls(mesh.x, mesh.y, mesh.vert, prob.node_id, prob.neq, prob.upresc, gamma=prob.gamma, **kw)

    def _check(self, rc, where):
        if rc:
            raise FemGpuError(rc, where)

    def close(self):
        if getattr(self, "_h", None):
            self._L.femgpu_euler_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        self._check(self._L.femgpu_euler_set_stream(self._h, _vp(stream_ptr)), "set_stream")

    def Build(self, u=None, du=None, want_matrix=False):
        """Build_M_K_F_SUPG from (u, du). Returns (R, Ae [nel, 144] or None)."""
        R = np.zeros(self.neq + 1)
        Ae = np.zeros((self.nel, 144)) if want_matrix else None
        uu = None if u is None else _f64(u)
        dd = None if du is None else _f64(du)
        self._check(self._L.femgpu_euler_build(self._h, _ptr(uu), _ptr(dd), _ptr(Ae), _ptr(R)), "Build")
        return R, Ae

    def precond_setup(self):
        """BlockDiag_precond_EBE_setup (blocks, inverses) or, CSR storage,
        ILUp_precond_setup (ILU(0) factors); then R := M^-1 R. Returns R."""
        R = np.zeros(self.neq + 1)
        self._check(self._L.femgpu_euler_precond_setup(self._h, _ptr(R)), "precond_setup")
        return R

    def set_amg(self, amg):
        """Use an :class:`AMG` context as the FEMGPU_PREC_AMG preconditioner
        of a CSR context (hierarchy rebuilt at every precond_setup)."""
        self._amg = amg
        self._check(self._L.femgpu_euler_set_amg(self._h, amg.handle), "set_amg")

    def scaling(self, want_matrix=False):
        """FemFunctions->scaling = Block_scaling_EBE after a Build: returns
        (R, Ae) scaled."""
        R = np.zeros(self.neq + 1)
        Ae = np.zeros(self.nel * 144) if want_matrix else None
        self._check(self._L.femgpu_euler_scale(self._h, _ptr(R), _ptr(Ae)), "scaling")
        return R, (Ae.reshape(self.nel, 144) if want_matrix else None)

    def set_slip(self, slip=None, cs=None, sn=None):
        """Slip walls: slip [nnodes] (the nodes with v1Type = -1) and the cosine
        and sine of their wall angles; None removes them."""
        if slip is None:
            self._check(self._L.femgpu_euler_set_slip(self._h, None, None, None), "set_slip")
            return
        self._slip = (_i32(slip), _f64(cs), _f64(sn))
        self._check(self._L.femgpu_euler_set_slip(self._h, *(_ptr(a) for a in self._slip)), "set_slip")

    def csr(self):
        """CSR storage: (IA, JA, CSR_by_Element [nel, 144], AA of the last build)."""
        nn = np.zeros(2, np.int32)
        self._check(self._L.femgpu_euler_csr(self._h, _ptr(nn), None, None, None, None), "csr")
        IA = np.zeros(int(nn[0]) + 1, np.int32)
        JA = np.zeros(max(int(nn[1]), 1), np.int32)
        sbe = np.zeros((self.nel, 144), np.int32)
        AA = np.zeros(int(nn[1]) + 1)
        self._check(self._L.femgpu_euler_csr(self._h, _ptr(nn), _ptr(IA), _ptr(JA), _ptr(sbe), _ptr(AA)), "csr")
        return IA, JA[: int(nn[1])], sbe, AA

    def solver(self, B=None, raise_on_nonconvergence=True):
        """pgmres (6-argument form) on the block EBE operator: X = A^-1 B
        (B None: the context's R). Returns (X, iterations)."""
        BB = None if B is None else _f64(B)
        X = np.zeros(self.neq + 1)
        it = ctypes.c_int(0)
        rc = self._L.femgpu_euler_solve(self._h, _ptr(BB), _ptr(X), ctypes.byref(it))
        if rc and (rc != -5 or raise_on_nonconvergence):
            raise FemGpuError(rc, "solver")
        return X, it.value

    def Predictor(self, u0, nsteps):
        """The time loop (Predictor_Old, or its BDF / TR-BDF2 form) for nsteps
        steps from u0. Returns (u after each stage [stages, neq+1], GMRES
        iterations [stages, ncorr]); a stage is a step, two per step for
        TR-BDF2."""
        u = np.array(u0, dtype=np.float64, copy=True)
        stages = nsteps * (2 if self.opts.method == 2 else 1)
        uh = np.zeros((stages, self.neq + 1))
        its = np.zeros((stages, self.opts.ncorr), np.int32)
        self._check(self._L.femgpu_euler_predictor(self._h, _ptr(u), int(nsteps), _ptr(uh), _ptr(its)),
                    "Predictor")
        return uh, its

    def set_bubbles(self, uB=None):
        """The DD build's element bubbles [nel, 4] for the following builds
        (None: zero)."""
        keep = None if uB is None else _f64(np.asarray(uB).reshape(-1))
        self._check(self._L.femgpu_euler_set_bubbles(self._h, None if keep is None else _ptr(keep)), "set_bubbles")

    def state(self):
        """The DD build's element bubbles [nel, 4] and each element's previous
        shock parameter delta_old [nel]."""
        uB = np.zeros((self.nel, 4))
        dold = np.zeros(self.nel)
        self._check(self._L.femgpu_euler_state(self._h, _ptr(uB), _ptr(dold)), "state")
        return uB, dold

    def predictor_dev(self, nsteps):
        """Predictor_Old continuing from the device state; returns the GMRES
        iterations [nsteps, ncorr]."""
        its = np.zeros((nsteps, self.opts.ncorr), np.int32)
        self._check(self._L.femgpu_euler_predictor_dev(self._h, int(nsteps), _ptr(its)), "predictor_dev")
        return its

    def last_times(self):
        """Seconds in (build, precond_setup, solve) of the last Predictor."""
        t = np.zeros(3)
        self._check(self._L.femgpu_euler_last_times(self._h, _ptr(t)), "last_times")
        return t

    def u_dev(self):
        return self._L.femgpu_euler_u_dev(self._h)


class NavierStokes:
    """Steady incompressible Navier-Stokes on one GPU: VMS/NSGS element build
    with bubble condensation, 3-dof block EBE storage with the nodal
    block-diagonal preconditioner, GMRES and the damped Newton loop
    (04_SS_NavierStokes_Equations/2D with StabilizationForm MS, EBE,
    BlockDiag).  ``Build``, ``precond_setup``, ``solver`` and ``Process``
    carry the names of the functions they replace; vectors have length
    neq+1."""

    def __init__(self, x, y, vert, node_id, neq, upresc, f=None, re=1000.0, velmax=1.0, precond="BlockDiag",
                 solver="GMRES", kmax=50, lmax=100, eta0=0.1, eta_case=2, tol_nl=1e-8, scheme="EBE",
                 ilu_blocks=0):
        L = load()
        o = NSOpts()
        L.femgpu_ns_default_opts(ctypes.byref(o))
        o.scheme = OPTS["scheme"][scheme.upper()]
        o.ilu_blocks = int(ilu_blocks)
        o.re, o.velmax = float(re), float(velmax)
        o.precond = OPTS["precond"][precond.upper()]
        o.solver = OPTS["solver"][solver.upper()]
        o.kmax, o.lmax, o.eta0, o.eta_case, o.tol_nl = int(kmax), int(lmax), float(eta0), int(eta_case), float(tol_nl)
        self.opts = o
        self._keep = [_f64(x), _f64(y), _i32(np.asarray(vert).reshape(-1)), _i32(np.asarray(node_id).reshape(-1)),
                      _f64(np.asarray(upresc).reshape(-1)),
                      None if f is None else _f64(np.asarray(f).reshape(-1))]
        self.nnodes = len(self._keep[0])
        self.nel = self._keep[2].size // 3
        self.neq = int(neq)
        h = _vp()
        rc = L.femgpu_ns_create(ctypes.byref(h), ctypes.byref(o), self.nnodes, _ptr(self._keep[0]),
                                _ptr(self._keep[1]), self.nel, _ptr(self._keep[2]), _ptr(self._keep[3]), self.neq,
                                _ptr(self._keep[4]), _ptr(self._keep[5]))
        if rc:
            raise FemGpuError(rc, "Preprocess")
        self._h = h
        self._L = L

    @classmethod
    def from_problem(cls, mesh, prob, **kw):
        return cls(mesh.x, mesh.y, mesh.vert, prob.node_id, prob.neq, prob.upresc, f=prob.f, re=prob.re,
                   velmax=prob.velmax, **kw)

    def _check(self, rc, where):
        if rc:
            raise FemGpuError(rc, where)

    def close(self):
        if getattr(self, "_h", None):
            self._L.femgpu_ns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        self._check(self._L.femgpu_ns_set_stream(self._h, _vp(stream_ptr)), "set_stream")

    def reset(self):
        self._check(self._L.femgpu_ns_reset(self._h), "reset")

    def Build(self, u=None, want_matrix=False):
        """Build_K_F_MS from u. Returns (F, Ae [nel, 81] or None)."""
        F = np.zeros(self.neq + 1)
        Ae = np.zeros((self.nel, 81)) if want_matrix else None
        uu = None if u is None else _f64(u)
        self._check(self._L.femgpu_ns_build(self._h, _ptr(uu), _ptr(Ae), _ptr(F)), "Build")
        return F, Ae

    def precond_setup(self):
        F = np.zeros(self.neq + 1)
        self._check(self._L.femgpu_ns_precond_setup(self._h, _ptr(F)), "precond_setup")
        return F


    def set_amg(self, amg):
        """Use an :class:`AMG` context as the FEMGPU_PREC_AMG preconditioner
        of a CSR context (hierarchy rebuilt at every precond_setup)."""
        self._amg = amg
        self._check(self._L.femgpu_ns_set_amg(self._h, amg.handle), "set_amg")
    def solver(self, B=None):
        BB = None if B is None else _f64(B)
        X = np.zeros(self.neq + 1)
        it = ctypes.c_int(0)
        rc = self._L.femgpu_ns_solve(self._h, _ptr(BB), _ptr(X), ctypes.byref(it))
        if rc and rc != -5:
            raise FemGpuError(rc, "solver")
        return X, it.value

    def csr(self):
        """CSR storage: (IA, JA, AA) of the last build."""
        nn = np.zeros(2, np.int32)
        self._check(self._L.femgpu_ns_csr(self._h, _ptr(nn), None, None, None), "csr")
        IA, JA, AA = np.zeros(nn[0] + 1, np.int32), np.zeros(nn[1], np.int32), np.zeros(nn[1] + 1)
        self._check(self._L.femgpu_ns_csr(self._h, _ptr(nn), _ptr(IA), _ptr(JA), _ptr(AA)), "csr")
        return IA, JA, AA

    def Process(self, maxit=2000):
        """Damped Newton from u = 0: (u, uhist [n, neq+1], |F| [n], w [n],
        GMRES iterations [n])."""
        u = np.zeros(self.neq + 1)
        uh = np.zeros((maxit, self.neq + 1))
        nF = np.zeros(maxit)
        w = np.zeros(maxit)
        g = np.zeros(maxit, np.int32)
        n = self._L.femgpu_ns_newton(self._h, int(maxit), _ptr(u), _ptr(uh), _ptr(nF), _ptr(w), _ptr(g))
        if n < 0:
            raise FemGpuError(n, "Process")
        return u, uh[:n], nF[:n], w[:n], g[:n]

    def u_dev(self):
        return self._L.femgpu_ns_u_dev(self._h)
