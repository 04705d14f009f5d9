"""Transient scalar transport (02_Transport_Equation/2D) on the GPU against
the reference's own run (tests/golden/tt_*.npz, generated by
oracle/ref_transient_harness.c from the reference's sources):

* the storage pattern and node numbering (CSR with or without SYMRCM, EDE);
* two consecutive Builds on a seeded state (u, a) -- Build_M_K_R_SUPG,
  Build_M_K_R_DD or Build_M_F_DD (with seeded bubbles), the DD builds' second
  build reading the first one's per-element shock parameter -- matrix storage
  and residual bit-identical;
* the reference's time loop (Predictor_Old, Predictor_Old_BDF,
  Predictor_Old_TRBDF2, Predictor_New, Predictor_New_BDF or
  Predictor_New_TRBDF2) from the problem's initial solution: u at the end of
  every multicorrection stage within 1e-8 relative, the same times and
  corrections per stage, GMRES iterations within 1 (the device reductions sum
  in another order).

Cases: CONE (CSR, SYMRCM, ILU(0), SUPG + CAU), CARTOLA (CSR, ILU(0), SUPG,
h_shock Option1, NORM multicorrection), CONE2 (CSR, SYMRCM, ILU(0), DD +
CAUDD; CSR, Diag, DD + CAU), CONE (EBE, Diag, DD + CAUDD, NORM) and PUDIM
(EDE, no preconditioner, SUPG + YZBeta, Option2, steady-state stop; 8 steps:
the device and reference runs agree to 4e-15 after the first step, and that
shock term amplifies the reductions' rounding differences about x3-5 per
step, past 1e-8 after 11 steps); BDF2
on CONE (CSR, SYMRCM, ILU(0)) and TR-BDF2 on CONE2 (DD + CAUDD) and CARTOLA
(EBE, Diag); Predictor_New with Build_M_F_DD (the element bubbles as unknowns
of the time loop) on CONE (CSR, SYMRCM, ILU(0), CAUDD) and CONE2 (EBE, Diag,
CAU, Option1, NORM); Predictor_New_BDF on CONE (CSR, SYMRCM, ILU(0), CAUDD)
and Predictor_New_TRBDF2 on CONE2 (EBE, Diag, CAU)."""
import ast
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "tt_*.npz")))
SOL_RTOL = 1e-8
# Condutivity / Reaction of the transient problems
# (02_Transport_Equation/2D/<P>/<P>_Condutivity.c, <P>_Reaction.c)
K_GAMMA = {"CONE": (1e-8, 0.0), "CONE2": (1e-8, 0.0), "CARTOLA": (1e-4, 2.0), "PUDIM": (1e-8, 0.0)}


def _context(g, c):
    import fem_codes_gb300 as fg
    k, gamma = K_GAMMA[c["problem"]]
    T = fg.SSTransport(g["x"], g["y"], g["node_type"], g["vert"], k, gamma, g["upresc"], beta=g["beta"],
                       fsrc=g["fsrc"], scheme=c["scheme"], reorder=c["reord"],
                       precond={"DIAG": "Diag"}.get(c["precond"].upper(), c["precond"]), shock=c["shock"],
                       hshock=c["hshock"], kmax=c["kmax"], lmax=c["lmax"], tol=c["tol"], solver="GMRES")
    T.set_transient(stab=c["stab"], alpha=c["alpha"], dt=c["dt"], final_time=c["final"], stop=c["stopmc"],
                    max_corr=c["max_corr"], nonlin_tol=c["nonlin_tol"], steady=c["steady"],
                    time_tol=c["time_tol"], method=c["tint"])
    return T


@pytest.mark.parametrize("name", CASES)
def test_transient_builds_and_predictor(gpu_lib, name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    c = ast.literal_eval(str(g["meta"]))
    neq = int(g["neq"])
    with _context(g, c) as T:
        assert T.neq == neq
        pat = T.pattern()
        assert np.array_equal(pat["node_id"], g["node_id"]), "node numbering"
        if c["scheme"] == "CSR":
            assert np.array_equal(pat["IA"], g["IA"]) and np.array_equal(pat["JA"], g["JA"]), "CSR pattern"
            assert np.array_equal(pat["sbe"], g["sbe"]), "CSR_by_Element"
        if c["tint"].upper().startswith("PREDICTOR2"):
            T.set_bubbles(g["ubB"], g["dubB"])
        R1, A1 = T.build_transient(g["ub"], g["dub"], want_matrix=True)
        assert np.array_equal(A1, g["A1"]), "first build: matrix"
        assert np.array_equal(R1[:neq], g["R1"][:neq]), "first build: residual"
        R2, A2 = T.build_transient(want_matrix=True)
        assert np.array_equal(A2, g["A2"]), "second build: matrix"
        assert np.array_equal(R2[:neq], g["R2"][:neq]), "second build: residual"
        # the reference asks its time criterion after every step but BDF's first
        bdf = c["tint"].upper() in ("PREDICTOR1_BDF", "PREDICTOR2_BDF")
        steps = int(g["tchecks"]) + (1 if bdf else 0)
        out = T.predictor(g["u0"], steps, iters_cap=64)
    assert len(out["t"]) == steps and len(out["ncorr"]) == int(g["stages"])
    assert np.array_equal(out["t"][1:] if bdf else out["t"], g["thist"])
    assert np.array_equal(out["ncorr"], g["ncorr"])
    ref = g["uhist"][:, :neq]
    err = np.abs(out["u"][:, :neq] - ref).max(axis=1) / np.maximum(np.abs(ref).max(axis=1), 1e-300)
    assert err.max() <= SOL_RTOL, err
    assert np.abs(out["iters"] - g["iters"]).max() <= 1
