"""CPU checks of the double-pairwise AMG preconditioner against the
reference's own AMG run on steady-transport matrices (tests/golden/amg_*.npz,
made by oracle/ref_amg_harness.c from amg_precond.c and CSR/AMG/*):

* the oracle's V-cycle (oracle/amg_oracle.c) on the reference's hierarchy
  reproduces AMG_precond and the AMG_precond_setup side effect F := M^-1 F
  bit for bit, and its AMG-preconditioned pgmres the reference's iterations
  and solution;
* the library's host set-up (matching_c / bcm_CSRMatrixHMatch and
  dpa_galerkin, host/amg.c, called through the C ABI without a GPU) rebuilds
  every level of the reference's hierarchy bit for bit."""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle

NAMES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "amg_*.npz")))


def load(name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    L = int(g["nlev"])
    levels = [(g[f"IA{l}"], g[f"JA{l}"], g[f"AA{l}"], g.get(f"rm{l}")) for l in range(L)]
    w = str(g["spec"]).split()
    return g, levels, dict(ncl=int(w[2]), beta=float(w[3]), omega=float(w[4]), nr=int(w[5]))


def test_fixtures_present():
    assert len(NAMES) >= 4


@pytest.mark.parametrize("name", NAMES)
def test_oracle_vcycle_bitexact(name):
    g, levels, p = load(name)
    assert len(levels) == 2 * p["ncl"] + 1
    assert np.array_equal(levels[0][0], g["IA"]) and np.array_equal(levels[0][2], g["AA"])
    for k in range(2):
        z = pyoracle.amg_vcycle(levels, p["omega"], p["nr"], g["q"][k])
        assert np.array_equal(z, g["z"][k]), f"V-cycle {k}"
    assert np.array_equal(pyoracle.amg_vcycle(levels, p["omega"], p["nr"], g["F"]), g["Fprec"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_amg_gmres_matches_reference(name):
    g, levels, p = load(name)
    X, it, Bp = pyoracle.amg_gmres(levels, p["omega"], p["nr"], g["F"], int(g["kmax"]), int(g["lmax"]),
                                   float(g["tol"]))
    assert np.array_equal(Bp, g["Fprec"])
    assert it == int(g["iters"])
    assert np.array_equal(X, g["X"])


def _lib():
    from fem_codes_gb300 import load as fg_load
    return fg_load()


@pytest.mark.parametrize("name", NAMES)
def test_host_setup_rebuilds_reference_hierarchy(name):
    L = _lib()
    g, levels, p = load(name)
    vp = ctypes.c_void_p
    ptr = lambda a: a.ctypes.data_as(vp)  # noqa: E731
    IA, JA, AA = (np.ascontiguousarray(a) for a in levels[0][:3])
    for l in range(len(levels) - 1):
        n = IA.size - 1
        rm = np.zeros(n + 1, np.int32)
        assert L.femgpu_dpa_match(n, ptr(IA), ptr(JA), ptr(AA), p["beta"], ptr(rm)) == 0
        assert np.array_equal(rm, levels[l][3]), f"matching of level {l}"
        nn = np.zeros(2, np.int32)
        assert L.femgpu_dpa_galerkin(n, ptr(IA), ptr(JA), ptr(AA), ptr(rm), ptr(nn), None, None, None) == 0
        IC, JC, AC = np.zeros(nn[0] + 1, np.int32), np.zeros(nn[1], np.int32), np.zeros(nn[1])
        assert L.femgpu_dpa_galerkin(n, ptr(IA), ptr(JA), ptr(AA), ptr(rm), ptr(nn), ptr(IC), ptr(JC),
                                     ptr(AC)) == 0
        assert np.array_equal(IC, levels[l + 1][0]), f"level {l + 1} IA"
        assert np.array_equal(JC, levels[l + 1][1]), f"level {l + 1} JA"
        assert np.array_equal(AC, levels[l + 1][2]), f"level {l + 1} AA"
        IA, JA, AA = IC, JC, AC


def test_host_setup_rejects_bad_input():
    L = _lib()
    vp = ctypes.c_void_p
    ptr = lambda a: a.ctypes.data_as(vp)  # noqa: E731
    IA = np.array([0, 2, 4], np.int32)
    JA = np.array([0, 5, 0, 1], np.int32)          # column out of range
    AA = np.ones(4)
    rm = np.zeros(3, np.int32)
    assert L.femgpu_dpa_match(2, ptr(IA), ptr(JA), ptr(AA), 0.25, ptr(rm)) == -1
    JA[1] = 1
    assert L.femgpu_dpa_match(2, ptr(IA), ptr(JA), ptr(AA), -0.5, ptr(rm)) == -1   # beta < 0, not -1
    assert L.femgpu_dpa_match(2, ptr(IA), ptr(JA), ptr(AA), 0.0, ptr(rm)) == 0
    bad = np.array([1, 1, 0], np.int32)            # not an involution
    nn = np.zeros(2, np.int32)
    assert L.femgpu_dpa_galerkin(2, ptr(IA), ptr(JA), ptr(AA), ptr(bad), ptr(nn), None, None, None) == -1
