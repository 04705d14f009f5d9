"""The C ABI library (CPU-side checks, no GPU): it builds, loads, exports every
entry point include/femgpu.h declares, and its host utilities (SYMRCM, ILU
level schedule) agree with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh


def declared_functions():
    src = open(os.path.join(ROOT, "include", "femgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(femgpu_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import fem_codes_gb300 as fg
    return fg.load()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_build_targets_sm103a_only():
    from fem_codes_gb300 import build as b
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_element_builds_compiled_without_contraction():
    """Translation units whose results must be bit-identical to the
    reference (element builds and block operators) are compiled with
    --fmad=false."""
    from fem_codes_gb300 import build as b
    assert {"amg.cu", "build.cu", "ebe_block.cu", "euler_build.cu", "ns_build.cu"} <= b.NO_FMA


def test_euler_bad_options_rejected_without_gpu(lib):
    import fem_codes_gb300 as fg
    o = fg.EulerOpts()
    lib.femgpu_euler_default_opts(ctypes.byref(o))
    assert (o.gamma, o.alpha, o.precond, o.solver, o.ncorr) == (1.4, 0.5, 3, 0, 2)
    o.ncorr = 0
    h = ctypes.c_void_p()
    x = np.zeros(3)
    v = np.zeros(3, np.int32)
    nid = np.zeros(12, np.int32)
    rc = lib.femgpu_euler_create(ctypes.byref(h), ctypes.byref(o), 3, x.ctypes.data, x.ctypes.data, 1,
                                 v.ctypes.data, nid.ctypes.data, 4, np.zeros(12).ctypes.data)
    assert rc == -1 and not h.value


def _pattern(nx, ny, perturb=0.0):
    m = structured_mesh(nx, ny, perturb=perturb)
    p = skew_problem(m)
    neq, node_id, lm = pyoracle.fill_lm(p.node_type, m.vert)
    IA, JA, _ = pyoracle.csr_pattern(neq, lm)
    return IA, JA


@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 1), (5, 3), (16, 16), (40, 20), (64, 64)])
def test_host_symrcm_matches_oracle(lib, nx, ny):
    IA, JA = _pattern(nx, ny, 0.1)
    n = IA.size - 1
    perm = np.zeros(n, np.int32)
    rc = lib.femgpu_symrcm(n, IA.ctypes.data_as(ctypes.c_void_p), JA.ctypes.data_as(ctypes.c_void_p),
                           perm.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    assert np.array_equal(perm, pyoracle.symrcm(IA, JA))


def test_host_symrcm_disconnected_components(lib):
    # block-diagonal pattern of two separate chains: the second component
    # starts at the lowest unvisited index (symrcm.c:71-77)
    rows = [[0, 1], [0, 1, 2], [1, 2], [3, 4], [3, 4]]
    IA = np.cumsum([0] + [len(r) for r in rows]).astype(np.int32)
    JA = np.concatenate(rows).astype(np.int32)
    perm = np.zeros(5, np.int32)
    lib.femgpu_symrcm(5, IA.ctypes.data_as(ctypes.c_void_p), JA.ctypes.data_as(ctypes.c_void_p),
                      perm.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(perm, pyoracle.symrcm(IA, JA))
    assert sorted(perm) == list(range(5))


def test_ilu_levels_natural_grid(lib):
    IA, JA = _pattern(32, 16)
    nl = lib.femgpu_ilu_levels(IA.size - 1, IA.ctypes.data_as(ctypes.c_void_p),
                               JA.ctypes.data_as(ctypes.c_void_p), 1)
    nu = lib.femgpu_ilu_levels(IA.size - 1, IA.ctypes.data_as(ctypes.c_void_p),
                               JA.ctypes.data_as(ctypes.c_void_p), 0)
    # unknowns form a 32 x 16 grid with 6-neighbour coupling: wavefront depth nx + ny - 1
    assert nl == 32 + 16 - 1
    assert nu == nl


def test_bad_arguments_rejected_without_gpu(lib):
    assert lib.femgpu_symrcm(0, None, None, None) == -1
    assert lib.femgpu_ilu_levels(-3, None, None, 1) == -1
    assert lib.femgpu_ilu_block_cut(0, None, None, 4, None, 0) == -1
    assert lib.femgpu_transport_ilu_blocks(None, None, 0) == -1


def test_block_cut_checks_capacity_and_pattern(lib):
    """femgpu_ilu_block_cut writes R + 1 = max(min(P, n), 1) + 1 ints: a
    buffer with less room, and patterns its level scan cannot read (a column
    out of range, columns not ascending, IA not starting at 0 or decreasing),
    are rejected before anything is written."""
    IA, JA = _pattern(12, 8)
    n = IA.size - 1
    vp = ctypes.c_void_p

    def cut(IA_, JA_, P, cap):
        first = np.full(cap + 1, -7, np.int32)
        rc = lib.femgpu_ilu_block_cut(IA_.size - 1, IA_.ctypes.data_as(vp), JA_.ctypes.data_as(vp), P,
                                      first.ctypes.data_as(vp), cap)
        return rc, first

    rc, first = cut(IA, JA, 4, 5)
    assert rc == 4 and first[0] == 0 and first[4] == n and first[5] == -7
    assert cut(IA, JA, 4, 4)[0] == -1                  # room for 4 boundaries, 5 needed
    assert cut(IA, JA, 0, 2)[0] == 1                   # P <= 0: one run, 2 ints
    assert cut(IA, JA, 0, 1)[0] == -1
    bad = JA.copy()
    bad[3] = -1
    assert cut(IA, bad, 4, 5)[0] == -1                 # negative column
    bad = JA.copy()
    bad[3] = n
    assert cut(IA, bad, 4, 5)[0] == -1                 # column past the last row
    r = next(i for i in range(n) if IA[i + 1] - IA[i] >= 2)
    bad = JA.copy()
    bad[IA[r]], bad[IA[r] + 1] = bad[IA[r] + 1], bad[IA[r]]
    assert cut(IA, bad, 4, 5)[0] == -1                 # columns not ascending
    badIA = IA.copy()
    badIA[0] = 1
    assert cut(badIA, JA, 4, 5)[0] == -1
    badIA = IA.copy()
    badIA[5] = badIA[4] - 1
    assert cut(badIA, JA, 4, 5)[0] == -1


def test_ns_bad_options_rejected_without_gpu(lib):
    """femgpu_ns_create validates its options before touching the device:
    storage / preconditioner pairs the reference's setPreconditioner.c
    rejects (BlockDiag needs EBE, ILU needs CSR), an unknown scheme, a bad
    forcing-term case."""
    import fem_codes_gb300 as fg
    x = np.zeros(3)
    v = np.zeros(3, np.int32)
    nid = np.zeros(9, np.int32)
    up = np.zeros(9)
    bad = [dict(scheme=2, precond=3), dict(scheme=0, precond=1), dict(scheme=1, precond=0),
           dict(eta_case=7), dict(kmax=0)]
    for kw in bad:
        o = fg.NSOpts()
        lib.femgpu_ns_default_opts(ctypes.byref(o))
        assert (o.scheme, o.precond, o.solver) == (0, 3, 0)
        for k, v_ in kw.items():
            setattr(o, k, v_)
        h = ctypes.c_void_p()
        rc = lib.femgpu_ns_create(ctypes.byref(h), ctypes.byref(o), 3, x.ctypes.data, x.ctypes.data, 1,
                                  v.ctypes.data, nid.ctypes.data, 3, up.ctypes.data, None)
        assert rc == -1 and not h.value, kw


def test_amg_and_transport_options_rejected_without_gpu(lib):
    """AMG parameters outside amg_precond.c's forms, and the transport's AMG
    preconditioner with EBE storage or a mixed precision, are refused before
    any device work."""
    import fem_codes_gb300 as fg
    h = ctypes.c_void_p()
    for ncl, beta, omega, nr in [(0, 0.25, 1.0, 2), (2, -0.5, 1.0, 2), (2, 0.25, 0.0, 2), (2, 0.25, 1.0, 0)]:
        assert lib.femgpu_amg_create(ctypes.byref(h), ncl, ctypes.c_double(beta), ctypes.c_double(omega), nr) == -1
    assert lib.femgpu_amg_setup(None, 1, None, None, None) == -1
    m = structured_mesh(4, 4)
    p = skew_problem(m)
    vert = np.ascontiguousarray(m.vert.reshape(-1), np.int32)
    nt = np.ascontiguousarray(p.node_type, np.int32)
    for scheme, precision in [(0, 0), (2, 1)]:
        o = fg.Opts()
        lib.femgpu_transport_default_opts(ctypes.byref(o))
        o.precond, o.scheme, o.precision, o.solver = 5, scheme, precision, 1
        t = ctypes.c_void_p()
        rc = lib.femgpu_transport_create(ctypes.byref(t), ctypes.byref(o), m.nnodes, m.x.ctypes.data,
                                         m.y.ctypes.data, nt.ctypes.data, m.nel, vert.ctypes.data,
                                         ctypes.c_double(p.k), ctypes.c_double(p.gamma), None,
                                         np.array([0.8, 0.5]).ctypes.data, None, p.upresc.ctypes.data)
        assert rc == -1 and not t.value, (scheme, precision)
