"""The reference-side shims (fem_codes_gb300/shims/): on the CPU.

* every shim compiles against its restated struct layout
  (-DFEMGPU_SHIM_OWN_TYPES), here and on any machine;
* where the reference tree exists: every restated struct has the size and
  every field the offset of the reference's own header (a generated C file
  of _Static_asserts over both headers), every shim compiles against the
  reference's own header, and each links into the reference's own driver loop
  -- the steady-transport Process.c, Predictor_Old.c and the Navier-Stokes
  Process.c -- into an executable with libfemgpu.  Without a GPU the
  transport and Euler executables run into the shim's error path, which
  prints and exits with status 1 as the reference does on a failure.

The GPU side (the shims reproducing the reference's golden runs) is
tests/test_gpu_shims.py."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIMS = os.path.join(ROOT, "fem_codes_gb300", "shims")
INC = os.path.join(ROOT, "include")
from __graft_entry__ import REFERENCE_DIR as REF  # noqa: E402
HAVE_REF = os.path.isdir(os.path.join(REF, "00_CommonFiles"))

# shim, restated-layout header, reference macro, reference header directory and header
FAMILIES = {
    "transport": ("femgpu_shim_transport.c", "shim_types_transport.h", "SSTranspEquation2D",
                  "01_SS_Transport_Equation/2D/01_CommonFiles", "SSTranspEquation.h"),
    "euler": ("femgpu_shim_euler.c", "shim_types_euler.h", "EulerEquations2D",
              "03_Euler_Equations/2D/01_CommonFiles", "EulerEquations.h"),
    "ns": ("femgpu_shim_ns.c", "shim_types_ns.h", "SSNavierStokesEquations2D",
           "04_SS_NavierStokes_Equations/2D/01_CommonFiles", "SSNavierStokesEquations.h"),
}


@pytest.fixture(scope="module")
def lib():
    import fem_codes_gb300 as fg
    return fg.load()


def _cc(args, cwd=None):
    r = subprocess.run(["gcc"] + args, capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.parametrize("fam", sorted(FAMILIES))
def test_shim_compiles_with_restated_layout(fam, tmp_path):
    shim = FAMILIES[fam][0]
    _cc(["-std=c11", "-Wall", "-Werror", "-Wno-unused-parameter", "-DFEMGPU_SHIM_OWN_TYPES", "-I" + SHIMS,
         "-I" + INC, "-c", os.path.join(SHIMS, shim), "-o", str(tmp_path / "shim.o")])


def struct_fields(header):
    """{struct name: [field names]} of a restated-layout header (every
    `typedef struct { ... } SHIM_T(Name);`)."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*SHIM_T\((\w+)\)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            fp = re.match(r".*?\(\s*\*\s*(\w+)\s*\)", decl)
            if fp:
                fields.append(fp.group(1))
                continue
            decl = re.sub(r"SHIM_T\(\w+\)", "T", decl)
            parts = decl.split(",")
            first = parts[0].split()
            parts[0] = first[-1]
            for p in parts:
                m = re.search(r"(\w+)\s*(\[[^\]]*\])?\s*$", p.replace("*", " "))
                fields.append(m.group(1))
        out[name] = fields
    return out


@pytest.mark.skipif(not HAVE_REF, reason="the reference tree is not present")
@pytest.mark.parametrize("fam", sorted(FAMILIES))
def test_restated_layout_matches_reference_header(fam, tmp_path):
    shim, types_h, macro, sub, hdr = FAMILIES[fam]
    structs = struct_fields(os.path.join(SHIMS, types_h))
    assert {"ParametersType", "MatrixDataType", "FemStructsType", "FemFunctionsType",
            "FemOtherFunctionsType", "NodeType", "ElementType"} <= set(structs)
    lines = [f'#include "{hdr}"', "#include <stddef.h>", "#define SHIM_T(n) own_##n",
             f'#include "{types_h}"']
    for name, fields in structs.items():
        lines.append(f"_Static_assert(sizeof(own_{name}) == sizeof({name}), \"sizeof {name}\");")
        for f in fields:
            lines.append(f"_Static_assert(offsetof(own_{name}, {f}) == offsetof({name}, {f}), \"{name}.{f}\");")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    _cc(["-std=gnu11", f"-D{macro}", "-w", "-I" + os.path.join(REF, sub), "-I" + SHIMS, "-c", str(src),
         "-o", str(tmp_path / "layout.o")])
    assert sum(len(f) for f in structs.values()) > 40


@pytest.mark.skipif(not HAVE_REF, reason="the reference tree is not present")
@pytest.mark.parametrize("fam", sorted(FAMILIES))
def test_shim_links_into_reference_driver_loop(fam, tmp_path, lib):
    shim, types_h, macro, sub, hdr = FAMILIES[fam]
    cf = os.path.join(REF, "00_CommonFiles")
    drv = os.path.join(REF, sub)
    blas = [os.path.join(cf, "BLAS_Operations", f + ".c") for f in ("daxpy", "ddot", "dcopy", "dzero", "dmax")]
    common = [os.path.join(cf, "Allocation_Operations", "mycalloc.c")] + blas
    if fam == "transport":
        extra = [os.path.join(drv, "Process.c")]
    elif fam == "euler":
        extra = [os.path.join(cf, "Time_Integration", "Predictor_Old.c")]
    else:
        extra = [os.path.join(drv, f) for f in ("Process.c", "eta_newton.c", "Coef_Lift_Drag.c", "eval_U.c",
                                                 "setzeros.c")] + [os.path.join(cf, "IO_Operations", "myfopen.c")]
    exe = tmp_path / f"drv_{fam}"
    libdir = os.path.join(ROOT, "fem_codes_gb300")
    cuda = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    _cc([f"-D{macro}", "-fcommon", "-w", "-I" + drv, "-I" + INC, "-I" + SHIMS, "-o", str(exe),
         os.path.join(ROOT, "tests", "shims", f"link_main_{fam}.c"), os.path.join(SHIMS, shim)] + extra + common +
        ["-L" + libdir, "-lfemgpu", "-L" + cuda, "-lcudart", "-Wl,-rpath," + libdir, "-lm"])
    if fam == "ns":
        return                               # its Process writes under ../03_output; linked, not run
    import torch
    if torch.cuda.is_available():
        return                               # the GPU run is tests/test_gpu_shims.py's
    r = subprocess.run([str(exe)], capture_output=True, text=True, cwd=tmp_path, timeout=120)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "femgpu shim: Build (context) failed" in r.stderr
