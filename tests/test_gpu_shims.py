"""The reference-side shims on the GPU: each shim is compiled here, against
the driver's struct layout (fem_codes_gb300/shims/shim_types_*.h, checked
field by field against the reference's headers in tests/test_shims.py),
together with a small driver of the reference's structs (tests/shims/) that
calls the installed function pointers in the order the reference's drivers
do.  Through the shims, the library reproduces the reference's own runs
(tests/golden): the steady-transport Picard run skew64_csr_ilu0_rcm (Build,
the restored precond_setup, 4-argument pgmres) and the Euler
predictor-multicorrector run eul_refletido_16x4 (Build, BlockDiag
precond_setup, 6-argument pgmres).

Bars: the first Build's RHS bit-identical, iterates to 1e-8 relative, GMRES
counts within one (the golden tests' bars)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIMS = os.path.join(ROOT, "fem_codes_gb300", "shims")
SOL_RTOL = 1e-8
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _driver(fam, tmp_path):
    libdir = os.path.join(ROOT, "fem_codes_gb300")
    out = str(tmp_path / f"libdrive_{fam}.so")
    cmd = ["gcc", "-shared", "-fPIC", "-O2", "-DFEMGPU_SHIM_OWN_TYPES", "-I" + SHIMS, "-I" + os.path.join(ROOT, "include"),
           "-o", out, os.path.join(ROOT, "tests", "shims", f"drive_{fam}.c"),
           os.path.join(SHIMS, f"femgpu_shim_{fam}.c"), "-L" + libdir, "-lfemgpu", "-Wl,-rpath," + libdir, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ctypes.CDLL(out)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_transport_shim_reproduces_reference_picard_run(gpu_lib, tmp_path):
    g, meta = load_golden("skew64_csr_ilu0_rcm")
    L = _driver("transport", tmp_path)
    f = L.drive_transport
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                  ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _ip]
    x, y = np.ascontiguousarray(g["x"]), np.ascontiguousarray(g["y"])
    # the driver's upresc plug-in is the SKEW rule; the golden holds the reference's values
    assert np.array_equal(np.where((x == 0.0) & (y > 0.3), 1.0, 0.0), g["upresc"])
    assert np.all(g["beta"] == g["beta"][0]) and np.all(g["fsrc"] == 0.0)
    neq, npic = int(g["neq"]), int(meta["npicard"])
    F1 = np.zeros(neq + 1)
    uh = np.zeros(npic * (neq + 1))
    its = np.zeros(npic, np.int32)
    rc = f(len(x), x, y, np.ascontiguousarray(g["node_type"], np.int32), len(g["vert"]),
           np.ascontiguousarray(g["vert"].reshape(-1), np.int32), 1e-4, 0.0, float(g["beta"][0, 0]),
           float(g["beta"][0, 1]), b"CSR", meta["reord"].encode(), b"ILU0", 30, 1000, 1e-8, npic, F1, uh, its)
    assert rc == neq, rc
    assert np.array_equal(F1, g["Ffirst"]), "RHS of the first Build"
    uh = uh.reshape(npic, neq + 1)
    for i in range(npic):
        assert _rel(uh[i, :-1], g["uhist"][i, :-1]) < SOL_RTOL, i
    assert np.all(np.abs(its - g["iters"]) <= 1), (its, g["iters"])


@pytest.mark.parametrize("scaling", [False, True])
def test_euler_shim_reproduces_reference_predictor_run(gpu_lib, tmp_path, scaling):
    """The reference's predictor loop through the shim's function pointers;
    with Scaling "BlockScaling" its scaling (Block_scaling_EBE) runs after
    each Build and the run follows the reference's scaled one."""
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "eul_refletido_16x4.npz")))
    L = _driver("euler", tmp_path)
    L.drive_euler_set_scaling(int(scaling))
    pre = "bs_" if scaling else ""
    f = L.drive_euler
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _ip, _ip, ctypes.c_int, _dp, ctypes.c_double,
                  ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                  ctypes.c_int, _dp, _ip]
    x, y = np.ascontiguousarray(g["x"]), np.ascontiguousarray(g["y"])
    nid = np.ascontiguousarray(g["node_id"].reshape(-1), np.int32)
    # the driver's REFLETIDO plug-ins give the reference's prescribed values
    left, bottom = np.abs(x) <= 1e-15, np.abs(y) <= 1e-15
    mine = np.stack([np.where(left, 1.0, 1.7), np.where(left, 2.9, 4.452878),
                     np.where(left | bottom, 0.0, -0.860744), np.where(left, 5.990715, 9.870181681)], 1)
    presc = g["node_id"].reshape(-1, 4) < 0
    assert np.array_equal(mine[presc], g["upresc"].reshape(-1, 4)[presc])
    neq, ns, nc = int(g["neq"]), int(g["nsteps"]), int(g["ncorr"])
    uh = np.zeros(ns * (neq + 1))
    its = np.zeros(ns * nc, np.int32)
    rc = f(len(x), x, y, len(g["vert"]), np.ascontiguousarray(g["vert"].reshape(-1), np.int32), nid, neq,
           np.ascontiguousarray(g["u0"]), float(g["alpha"]), float(g["dt"]), float(g["stab_tol"]), int(g["kmax"]),
           int(g["lmax"]), float(g["tol"]), ns, nc, uh, its)
    assert rc == 0, rc
    uh = uh.reshape(ns, neq + 1)
    ref = g[pre + "uhist"].reshape(ns, neq + 1)
    assert np.abs(uh - ref).max() / np.abs(ref).max() < SOL_RTOL
    assert np.abs(its - g[pre + "iters"].reshape(-1)).max() <= 1, (its, g[pre + "iters"])
