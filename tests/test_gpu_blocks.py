"""GPU parity of the multi-dof EBE operators (Euler ndof 4, Navier-Stokes
ndof 3) against the reference's own outputs (tests/golden/blk_*.npz) --
bit-identical -- and against the oracle on a larger mesh."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle
from fem_codes_gb300.mesh import structured_mesh

pytestmark = pytest.mark.gpu

_vp = ctypes.c_void_p


def _p(a):
    return a.ctypes.data_as(_vp) if a is not None else None


def bind(L):
    for name, args in {
        "femgpu_ebe_create": [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int],
        "femgpu_ebe_set_matrix": [_vp, _vp],
        "femgpu_ebe_matvec": [_vp, _vp, _vp],
        "femgpu_ebe_matvec2": [_vp, _vp, _vp, ctypes.c_int],
        "femgpu_ebe_blockdiag_setup": [_vp, _vp, _vp, _vp],
        "femgpu_ebe_blockdiag_apply": [_vp, _vp, _vp],
    }.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = ctypes.c_int
    L.femgpu_ebe_destroy.argtypes = [_vp]
    L.femgpu_ebe_destroy.restype = None
    return L


def gpu_block_ops(L, ndof, nnodes, vert, node_id, neq, A, P, p, F):
    h = _vp()
    vert = np.ascontiguousarray(vert, np.int32).reshape(-1)
    node_id = np.ascontiguousarray(node_id, np.int32).reshape(-1)
    assert L.femgpu_ebe_create(ctypes.byref(h), ndof, nnodes, vert.size // 3, _p(vert), _p(node_id), neq) == 0
    try:
        A = np.ascontiguousarray(A, np.float64)
        assert L.femgpu_ebe_set_matrix(h, _p(A)) == 0
        out = {}
        Q = np.zeros(neq + 1)
        assert L.femgpu_ebe_matvec(h, _p(np.array(P, dtype=np.float64)), _p(Q)) == 0
        out["Q"] = Q
        d2 = ndof * ndof
        BD, invBD = np.zeros(nnodes * d2), np.zeros(nnodes * d2)
        Fo = np.array(F, dtype=np.float64)
        assert L.femgpu_ebe_blockdiag_setup(h, _p(Fo), _p(BD), _p(invBD)) == 0
        out.update(F=Fo, BD=BD.reshape(nnodes, d2), invBD=invBD.reshape(nnodes, d2))
        Z = np.zeros(neq + 1)
        pp = np.array(p, dtype=np.float64)
        assert L.femgpu_ebe_blockdiag_apply(h, _p(pp), _p(Z)) == 0
        Z[neq] = 0.0
        out["Z"] = Z
        if ndof == 4:
            for key, inv in (("Q2", 1), ("Q2no", 0)):
                Qx = np.zeros(neq + 1)
                assert L.femgpu_ebe_matvec2(h, _p(np.array(P, dtype=np.float64)), _p(Qx), inv) == 0
                out[key] = Qx
        return out
    finally:
        L.femgpu_ebe_destroy(h)


@pytest.mark.parametrize("name", ["blk_euler_10x6", "blk_ns_9x7"])
def test_block_ops_bitexact_vs_reference(gpu_lib, name):
    L = bind(gpu_lib)
    g = dict(np.load(f"{GOLDEN}/{name}.npz"))
    ndof, neq = int(g["ndof"]), int(g["neq"])
    out = gpu_block_ops(L, ndof, len(g["x"]), g["vert"], g["node_id"], neq, g["A"], g["P"], g["p"], g["F0"])
    g["Z"][neq] = 0.0
    for key in ["Q", "BD", "invBD", "F", "Z"] + (["Q2", "Q2no"] if ndof == 4 else []):
        assert np.array_equal(out[key], g[key]), f"{name}: {key}"


@pytest.mark.parametrize("ndof", [3, 4])
def test_block_ops_vs_oracle_large(gpu_lib, ndof):
    L = bind(gpu_lib)
    m = structured_mesh(120, 80, perturb=0.2, seed=5)
    rng = np.random.default_rng(ndof)
    presc = (rng.random((m.nnodes, ndof)) < 0.05) | (m.x == 0.0)[:, None]
    node_id = np.full((m.nnodes, ndof), -1, np.int32)
    neq = int((~presc).sum())
    node_id[~presc] = np.arange(neq, dtype=np.int32)
    mm = 3 * ndof
    A = rng.uniform(-1, 1, (m.nel, mm * mm)) + np.eye(mm).reshape(-1)[None] * 4.0
    P = rng.uniform(-1, 1, neq + 1); P[neq] = 0.0
    p = rng.uniform(-1, 1, neq + 1); p[neq] = 0.0
    F = rng.uniform(-1, 1, neq + 1); F[neq] = 0.0
    ref = pyoracle.block_ops(ndof, m.nnodes, m.vert, node_id, neq, A, P, p, F)
    out = gpu_block_ops(L, ndof, m.nnodes, m.vert, node_id, neq, A, P, p, F)
    ref["Z"][neq] = 0.0
    for key in ["Q", "BD", "invBD", "F", "Z"] + (["Q2", "Q2no"] if ndof == 4 else []):
        assert np.array_equal(out[key], ref[key]), key
