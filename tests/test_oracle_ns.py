"""The oracle's restatement of the steady Navier-Stokes VMS build
(Build_K_F_MS.c) and damped Newton (Process.c, eta_newton.c) against the
reference's own outputs (tests/golden/ns_*.npz): bit-identical element
matrices, residuals, stabilisation state, Newton iterates, residual norms,
damping factors and GMRES iteration counts."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle

CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "ns_*.npz")))


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _args(g):
    return (g["x"], g["y"], g["vert"], g["node_id"], int(g["neq"]), g["upresc"], g["f"], float(g["re"]),
            float(g["velmax"]))


@pytest.mark.parametrize("name", CASES)
def test_ns_builds_bitexact(name):
    g = _load(name)
    Ae, F, dold, nold = pyoracle.ns_builds(*_args(g), g["us"])
    for b in range(len(g["us"])):
        assert np.array_equal(Ae[b], g["Ae"][b]), b
        assert np.array_equal(F[b], g["F"][b]), b
    assert np.array_equal(dold, g["delta_old"])
    assert np.array_equal(nold, g["normres_old"])


@pytest.mark.parametrize("name", CASES)
def test_ns_newton_bitexact(name):
    g = _load(name)
    uh, nF, w, its = pyoracle.ns_newton(*_args(g), kmax=int(g["kmax"]), lmax=int(g["lmax"]), eta0=float(g["eta0"]),
                                        ecase=int(g["ecase"]), tolnl=float(g["tolnl"]), maxit=int(g["maxit"]))
    assert len(nF) == len(g["normF"])
    assert np.array_equal(its, g["gmres"])
    assert np.array_equal(w, g["w"])
    assert np.array_equal(nF, g["normF"])
    assert np.array_equal(uh, g["uhist"])
