import ast
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Conductivity / reaction of the problems used by the golden cases
# (01_SS_Transport_Equation/2D/<PROBLEM>/<PROBLEM>_Condutivity.c, _Reaction.c).
PROBLEM_K_GAMMA = {"SKEW": (1e-4, 0.0), "CONVECTION": (1e-7, 0.0), "REACTION": (1e-6, 1.0),
                   "HEMKER": (1e-4, 0.0), "VALIDACAO": (1.0, 1.0)}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    """Steady-transport golden cases (blk_* hold block operators, eul_* the
    Euler build and predictor, ns_* the Navier-Stokes build and Newton,
    amg_* the AMG hierarchy and V-cycle, vtu_* the reference's VTU output,
    tt_* the transient transport builds and time loop)."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith(("amg_", "blk_", "eul_", "ns_", "vtu_", "tt_")))


def load_golden(name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = ast.literal_eval(str(g["meta"]))
    return g, meta


def run_kwargs(meta):
    """Map a golden case's harness options to solver keyword arguments."""
    m = dict(meta)
    m.pop("problem", None)
    return dict(scheme=m.get("scheme", "CSR"), reord=m.get("reord", "NOT"),
                precond=m.get("precond", "ILU0"), shock=m.get("shock", "CAU"),
                hshock=m.get("hshock", "2sqrtArea"), outflow=m.get("outflow", "NOT"),
                kmax=m.get("kmax", 30), lmax=m.get("lmax", 1000), tol=m.get("tol", 1e-8),
                npicard=m.get("npicard", 3))


@pytest.fixture(scope="session")
def gpu_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fem_codes_gb300 as fg
    return fg.load()
