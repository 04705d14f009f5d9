"""GPU parity of the 2D Euler path (Build_M_K_F_SUPG + Delta_CAU element
build, BlockDiag precond_setup, pgmres on the block EBE operator,
Predictor_Old) against the reference's own outputs (tests/golden/eul_*.npz)
and against the oracle on larger meshes.

Bars: element matrices, residuals and the preconditioned residual are
bit-identical (same operation order, no FMA contraction).  Solutions after
GMRES agree to a relative 1e-8: the device reductions sum dot products in a
different order than the reference's ddot, so the Krylov iterates differ in
the last bits."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle
from fem_codes_gb300.mesh import euler_cfl_dt, refletido_problem, structured_mesh

pytestmark = pytest.mark.gpu

CASES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "eul_*.npz")))
SOL_RTOL = 1e-8


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _euler(g, **kw):
    import fem_codes_gb300 as fg
    args = dict(gamma=float(g["gamma"]), alpha=float(g["alpha"]), dt=float(g["dt"]),
                stab_tol=float(g["stab_tol"]), kmax=int(g["kmax"]), lmax=int(g["lmax"]), tol=float(g["tol"]),
                ncorr=int(g["ncorr"]))
    args.update(kw)
    return fg.Euler(g["x"], g["y"], g["vert"], g["node_id"], int(g["neq"]), g["upresc"], **args)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_euler_build_bitexact_vs_reference(gpu_lib, name):
    g = _load(name)
    with _euler(g) as eu:
        R, Ae = eu.Build(g["u"], g["du"], want_matrix=True)
    assert np.array_equal(Ae, g["Ae"])
    assert np.array_equal(R, g["R"])


@pytest.mark.parametrize("name", CASES)
def test_euler_build_slip_walls_bitexact_vs_reference(gpu_lib, name):
    """Slip walls (v1Type = -1 on the bottom wall): the rotation of
    Build_M_K_F_SUPG.c:1044-1056 / rotation.c, element matrices and residual
    bit-identical to the reference's build; removing the walls restores the
    unrotated build."""
    g = _load(name)
    with _euler(g) as eu:
        eu.set_slip(g["slip"], g["slip_cs"], g["slip_sn"])
        R, Ae = eu.Build(g["u"], g["du"], want_matrix=True)
        assert np.array_equal(Ae, g["slip_Ae"])
        assert np.array_equal(R, g["slip_R"])
        eu.set_slip(None)
        R, Ae = eu.Build(g["u"], g["du"], want_matrix=True)
    assert np.array_equal(Ae, g["Ae"]) and np.array_equal(R, g["R"])


@pytest.mark.parametrize("name", CASES)
def test_euler_precond_setup_bitexact(gpu_lib, name):
    """R := D^-1 R after the build (BlockDiag_precond_EBE_setup.c:82)."""
    g = _load(name)
    neq = int(g["neq"])
    ref = pyoracle.block_ops(4, len(g["x"]), g["vert"], g["node_id"], neq, g["Ae"], np.zeros(neq + 1),
                             np.zeros(neq + 1), g["R"])
    with _euler(g) as eu:
        eu.Build(g["u"], g["du"])
        Rp = eu.precond_setup()
    assert np.array_equal(Rp[:neq], ref["F"][:neq])


@pytest.mark.parametrize("name", CASES)
def test_euler_predictor_vs_reference(gpu_lib, name):
    g = _load(name)
    with _euler(g) as eu:
        uh, its = eu.Predictor(g["u0"], int(g["nsteps"]))
    assert _rel(uh, g["uhist"]) < SOL_RTOL
    assert np.abs(its.astype(int) - g["iters"].astype(int)).max() <= 1


@pytest.mark.parametrize("name", CASES)
def test_euler_block_scaling_vs_reference(gpu_lib, name):
    """Scaling "BlockScaling" (Block_scaling_EBE after every Build,
    Predictor_Old.c:73): the scaled element matrices and R bit-identical to
    the reference's, and its predictor-multicorrector run within 1e-8."""
    g = _load(name)
    with _euler(g) as eu:
        eu.Build(g["u"], g["du"])
        R, Ae = eu.scaling(want_matrix=True)
    assert np.array_equal(Ae, g["bs_Ae"])
    assert np.array_equal(R, g["bs_R"])
    with _euler(g, scaling="BlockScaling") as eu:
        uh, its = eu.Predictor(g["u0"], int(g["nsteps"]))
    assert _rel(uh, g["bs_uhist"]) < SOL_RTOL
    assert np.abs(its.astype(int) - g["bs_iters"].astype(int)).max() <= 1


def test_euler_build_large_vs_oracle(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(96, 24, lx=4.0, ly=1.0, perturb=0.25, seed=11)
    pb = refletido_problem(m)
    rng = np.random.default_rng(5)
    u = pb.u0 * (1.0 + 0.08 * rng.uniform(-1, 1, pb.neq + 1))
    du = 0.2 * rng.uniform(-1, 1, pb.neq + 1)
    u[pb.neq] = du[pb.neq] = 0.0
    dt = euler_cfl_dt(m, 5.0)
    Ao, Ro = pyoracle.euler_build(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, u, du, alpha=0.5, dt=dt,
                                  stab_tol=1e-6)
    with fg.Euler.from_problem(m, pb, alpha=0.5, dt=dt, stab_tol=1e-6) as eu:
        R, Ae = eu.Build(u, du, want_matrix=True)
    assert np.array_equal(Ae, Ao)
    assert np.array_equal(R, Ro)


def test_euler_dimensionless_vs_oracle(gpu_lib):
    """dimensionless_Ax_Ay_calculations (Ax_Ay_calculations.c:3-52)."""
    import fem_codes_gb300 as fg
    m = structured_mesh(20, 6, lx=4.0, ly=1.0, perturb=0.2, seed=2)
    pb = refletido_problem(m)
    rng = np.random.default_rng(9)
    u = pb.u0 * (1.0 + 0.05 * rng.uniform(-1, 1, pb.neq + 1))
    du = 0.1 * rng.uniform(-1, 1, pb.neq + 1)
    u[pb.neq] = du[pb.neq] = 0.0
    Ao, Ro = pyoracle.euler_build(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, u, du, alpha=0.5, dt=0.01,
                                  stab_tol=1e-6, mach=0.8, dimensionless=True)
    with fg.Euler.from_problem(m, pb, alpha=0.5, dt=0.01, stab_tol=1e-6, mach=0.8, dimensionless=True) as eu:
        R, Ae = eu.Build(u, du, want_matrix=True)
    assert np.array_equal(Ae, Ao)
    assert np.array_equal(R, Ro)


def test_euler_predictor_large_vs_oracle(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(64, 16, lx=4.0, ly=1.0)
    pb = refletido_problem(m)
    dt = euler_cfl_dt(m, 5.0)
    uo, ito = pyoracle.euler_predictor(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, pb.u0, 3, 2, dt=dt,
                                       kmax=30, lmax=100, tol=1e-8)
    with fg.Euler.from_problem(m, pb, dt=dt, kmax=30, lmax=100, tol=1e-8, ncorr=2) as eu:
        uh, its = eu.Predictor(pb.u0, 3)
    assert _rel(uh, uo) < SOL_RTOL
    assert np.abs(its.astype(int) - ito.astype(int)).max() <= 1


def test_euler_fgmres_matches_pgmres(gpu_lib):
    """Right-preconditioned FGMRES (stops on the true residual) reaches the
    same corrector solutions as the reference's left-preconditioned GMRES
    when both solve tightly."""
    g = _load(CASES[0])
    with _euler(g, tol=1e-12, lmax=200) as a, _euler(g, tol=1e-12, lmax=200, solver="FGMRES") as b:
        ua, _ = a.Predictor(g["u0"], 2)
        ub, _ = b.Predictor(g["u0"], 2)
    assert _rel(ub, ua) < 1e-7


MIXED_RTOL = 1e-6   # mixed vs FP64 precision, same solver and criterion (relative, max norm)
RULE_RTOL = 5e-5    # true-residual (FGMRES) vs the reference's preconditioned-residual stop, both at 1e-8


def test_euler_mixed_precision_vs_fp64_and_oracle(gpu_lib):
    """FP32 element matrices and block-diagonal preconditioner inside FGMRES,
    each restart from the FP64 residual and each solve accepted on the FP64
    residual (1e-8): the predictor states stay within MIXED_RTOL of the FP64
    FGMRES run, and both within RULE_RTOL of the FP64 oracle (the reference's
    left-preconditioned GMRES, whose 1e-8 applies to ||D^-1 r||)."""
    import fem_codes_gb300 as fg
    m = structured_mesh(64, 16, lx=4.0, ly=1.0)
    pb = refletido_problem(m)
    dt = euler_cfl_dt(m, 5.0)
    uo, _ = pyoracle.euler_predictor(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, pb.u0, 3, 2, dt=dt,
                                     kmax=30, lmax=100, tol=1e-8)
    kw = dict(dt=dt, kmax=30, lmax=100, tol=1e-8, ncorr=2, solver="FGMRES")
    with fg.Euler.from_problem(m, pb, precision="MIXED_IR", **kw) as eu:
        um, its = eu.Predictor(pb.u0, 3)
    with fg.Euler.from_problem(m, pb, precision="FP64", **kw) as eu:
        u64, _ = eu.Predictor(pb.u0, 3)
    assert _rel(um, u64) < MIXED_RTOL
    assert _rel(u64, uo) < RULE_RTOL
    assert _rel(um, uo) < RULE_RTOL
    assert (its > 0).all()


def test_euler_mixed_precision_needs_fgmres(gpu_lib):
    import fem_codes_gb300 as fg
    g = _load(CASES[0])
    with pytest.raises(fg.FemGpuError) as ei:
        _euler(g, precision="MIXED_IR")
    assert ei.value.code == -1


def test_euler_call_order(gpu_lib):
    import fem_codes_gb300 as fg
    g = _load(CASES[0])
    with _euler(g) as eu:
        with pytest.raises(fg.FemGpuError) as ei:
            eu.precond_setup()
        assert ei.value.code == -9


@pytest.mark.parametrize("name", CASES)
def test_euler_csr_build_and_ilu0_setup_bitexact(gpu_lib, name):
    """CSR storage (the Euler driver's csr_Initialization.c / csr_assembly.c,
    setMatrixVectorProductType.c:24) with ILU(0) (setPreconditioner.c:
    118-128): pattern, CSR_by_Element slots, the assembled values and the
    residual of a Build, and R := M^-1 R of precond_setup, all bit-identical
    to the reference's."""
    g = _load(name)
    with _euler(g, scheme="CSR", precond="ILU0") as eu:
        R, _ = eu.Build(g["u"], g["du"])
        IA, JA, sbe, AA = eu.csr()
        Rp = eu.precond_setup()
    assert np.array_equal(IA, g["csr_IA"]) and np.array_equal(JA, g["csr_JA"])
    assert np.array_equal(sbe, g["csr_sbe"])
    assert np.array_equal(AA, g["csr_AA"])
    assert np.array_equal(R, g["csr_R"])
    assert np.array_equal(Rp, g["csr_Rp"])


@pytest.mark.parametrize("name", CASES)
def test_euler_csr_ilu0_predictor_vs_reference(gpu_lib, name):
    """Predictor_Old with CSR storage and ILU(0)-GMRES against the
    reference's run: iterates to 1e-8, GMRES counts within one."""
    g = _load(name)
    with _euler(g, scheme="CSR", precond="ILU0") as eu:
        uh, its = eu.Predictor(g["u0"], int(g["nsteps"]))
    assert _rel(uh, g["csr_uhist"]) < SOL_RTOL
    assert np.abs(its.astype(int) - g["csr_iters"].astype(int)).max() <= 1


def test_euler_csr_block_ilu0_fgmres_converges(gpu_lib):
    """Block ILU(0) over 8 row blocks of the 4-dof CSR system with FGMRES
    (accepted on the true residual): the predictor's states stay within the
    solver tolerance's reach of the FP64 ILU(0)-GMRES run."""
    import fem_codes_gb300 as fg
    m = structured_mesh(64, 16, lx=4.0, ly=1.0)
    pb = refletido_problem(m)
    dt = euler_cfl_dt(m, 5.0)
    kw = dict(dt=dt, kmax=50, lmax=100, tol=1e-10, ncorr=2, scheme="CSR", precond="ILU0")
    with fg.Euler.from_problem(m, pb, **kw) as eu:
        ref, _ = eu.Predictor(pb.u0, 3)
    with fg.Euler.from_problem(m, pb, solver="FGMRES", ilu_blocks=8, **kw) as eu:
        uh, its = eu.Predictor(pb.u0, 3)
    assert np.all(its > 0)
    assert _rel(uh, ref) < 1e-6


@pytest.mark.parametrize("name", CASES)
def test_euler_csr_amg_setup_bitexact(gpu_lib, name):
    """CSR storage with the AMG preconditioner (setPreconditioner.c:130-140 of
    the Euler driver): R := M^-1 R of precond_setup equals the reference's
    AMG_precond_setup on the same CSR system bit for bit."""
    import fem_codes_gb300 as fg
    g = _load(name)
    _, _, ncl, beta, omega, nr = str(g["amg_spec"]).split()
    amg = fg.AMG(ncl=int(ncl), beta=float(beta), omega=float(omega), nr=int(nr))
    neq = int(g["neq"])
    try:
        with _euler(g, scheme="CSR", precond="AMG") as eu:
            eu.set_amg(amg)
            eu.Build(g["u"], g["du"])
            Rp = eu.precond_setup()
    finally:
        amg.close()
    assert np.array_equal(Rp[:neq], g["amg_Fp"])


@pytest.mark.parametrize("name", CASES)
def test_euler_yzbeta_vs_reference(gpu_lib, name):
    """ShockCapture "YZBeta" (Delta_YZBeta.c:6-108, setStabilizationForm.c:27)
    with the deck's Y^-1: two consecutive Builds from a zero delta_old, the
    second blending the first's per-element delta, bit-identical Ae and R;
    the predictor-multicorrector run (delta_old zeroed at its start, as
    Predictor_Old.c:23 allocates it) within 1e-8."""
    g = _load(name)
    with _euler(g, shock="YZBeta", invY=g["yz_invY"]) as eu:
        R1, Ae1 = eu.Build(g["u"], g["du"], want_matrix=True)
        R2, Ae2 = eu.Build(g["u"], g["du"], want_matrix=True)
    assert np.array_equal(Ae1, g["yz_Ae1"]) and np.array_equal(R1, g["yz_R1"])
    assert np.array_equal(Ae2, g["yz_Ae2"]) and np.array_equal(R2, g["yz_R2"])
    with _euler(g, shock="YZBeta", invY=g["yz_invY"]) as eu:
        uh, its = eu.Predictor(g["u0"], int(g["nsteps"]))
    assert _rel(uh, g["yz_uhist"]) < SOL_RTOL
    assert np.abs(its.astype(int) - g["yz_iters"].astype(int)).max() <= 1


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("method,key,nsteps", [("Predictor1_BDF", "bdf", 4), ("Predictor1_TRBDF2", "tr", 2)])
def test_euler_bdf_trbdf2_vs_reference(gpu_lib, name, method, key, nsteps):
    """TimeIntegration Predictor1_BDF (Predictor_Old_BDF.c: an implicit first
    step, then BDF2) and Predictor1_TRBDF2 (Predictor_Old_TRBDF2.c: a TR and
    a BDF2 stage per step, the build's DeltaT switching from the TR to the
    BDF2 sub-step at the first BDF2 stage) against the reference's own loops
    (oracle/ref_euler_harness.c): u after every stage within 1e-8, GMRES
    iterations within 1."""
    g = _load(name)
    with _euler(g, method=method) as eu:
        uh, its = eu.Predictor(g["u0"], nsteps)
    ref = g[key + "_uhist"]
    assert uh.shape == ref.shape
    assert _rel(uh, ref) < SOL_RTOL, _rel(uh, ref)
    assert np.abs(its.astype(int) - g[key + "_iters"].astype(int)).max() <= 1



@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("shock,key", [("CAUDD", "dd"), ("YZBeta", "ddyz")])
def test_euler_dd_build_vs_reference(gpu_lib, name, shock, key):
    """StabilizationForm "DD" (Build_M_K_F_DD_Transiente.c: bubble-enriched
    element, the bubble condensed into the 12x12 element matrix and the
    element bubble updated in the build) with Delta_DD (CAUDD) or
    Delta_YZBeta: two consecutive Builds from the same seeded bubbles and a
    zero delta_old as the reference's own; R, the bubbles and delta_old
    and Ae bit-identical.  (The reference's Ax_Ay_calculations never sets
    Ay[0][3], which this build reads; the reference library is compiled
    with zero-filled locals, so it reads the Jacobian's structural 0 there,
    as the device build does.)"""
    g = _load(name)
    invY = g["yz_invY"] if shock == "YZBeta" else (1.0, 1.0, 1.0, 1.0)
    with _euler(g, stab="DD", shock=shock, invY=invY) as eu:
        eu.set_bubbles(g["dd_uB0"].reshape(-1, 4))
        R1, Ae1 = eu.Build(g["u"], g["du"], want_matrix=True)
        R2, Ae2 = eu.Build(g["u"], g["du"], want_matrix=True)
        uB, dold = eu.state()
    assert np.array_equal(R1, g[key + "_R1"]) and np.array_equal(R2, g[key + "_R2"])
    assert np.array_equal(Ae1, g[key + "_Ae1"]) and np.array_equal(Ae2, g[key + "_Ae2"])
    assert np.array_equal(uB.reshape(-1), g[key + "_uB"])
    assert np.array_equal(dold, g[key + "_dold"])


@pytest.mark.parametrize("name", CASES)
def test_euler_dd_predictor_vs_reference(gpu_lib, name):
    """Predictor_Old with the DD build and Delta_DD (bubbles and delta_old
    zero at the start) against the reference's own run: u after every step
    within 1e-8, GMRES iterations within 1."""
    g = _load(name)
    with _euler(g, stab="DD", shock="CAUDD") as eu:
        uh, its = eu.Predictor(g["u0"], int(g["nsteps"]))
    assert _rel(uh, g["dd_uhist"]) < SOL_RTOL, _rel(uh, g["dd_uhist"])
    assert np.abs(its.astype(int) - g["dd_iters"].astype(int)).max() <= 1


def test_euler_dd_options_checked(gpu_lib):
    """The DD build takes CAUDD or YZBeta; CAUDD is refused with SUPG, and
    the plain CAU with DD (setStabilizationForm.c pairs them that way)."""
    import fem_codes_gb300 as fg
    g = _load(CASES[0])
    for kw in (dict(stab="SUPG", shock="CAUDD"), dict(stab="DD", shock="CAU")):
        with pytest.raises(fg.FemGpuError):
            _euler(g, **kw)
