"""GPU parity at the benchmark configurations themselves, against the CPU
oracle (which reproduces the reference's own outputs bit for bit on every
golden fixture):

* the 2048x1024 transport mesh (4,194,304 triangles, interior nodes perturbed
  by +-0.2h, seed 1234, SYMRCM): CSR pattern, CSR_by_Element slot map, the
  SYMRCM renumbering (node ids), the first Build's matrix and RHS, one CSR
  matvec, the ILU(0) precond_setup F := M^-1 F and one ILU(0) application --
  all bit-identical;
* the 1024x256 Euler REFLETIDO mesh (524,288 triangles): the element
  Jacobians Ae and the residual R of Build_M_K_F_SUPG, bit-identical;
* two FP64 time steps of the predictor-multicorrector on the 256x64 Euler
  mesh, within 1e-8 of the oracle's run.

The oracle needs a few seconds of one CPU core for each of these."""
import numpy as np
import pytest

from oracle import pyoracle
from fem_codes_gb300.mesh import euler_cfl_dt, refletido_problem, skew_problem, structured_mesh

pytestmark = pytest.mark.gpu

SOL_RTOL = 1e-8


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check_fused_product(T, pat, A, P, Qref):
    """The FGMRES operator (fused multiply-adds, one rounding per entry)
    against csrmv.c's separately rounded sums: each row within
    2 nnz_row eps of sum |a_ij p_j|."""
    import ctypes
    import torch
    vp = ctypes.c_void_p
    IAd, JAd, AAd = T.csr_dev()
    Pd = torch.from_numpy(np.ascontiguousarray(P)).cuda()
    Qd = torch.zeros_like(Pd)
    torch.cuda.synchronize()
    assert T._L.femgpu_csrmv_f64_fused(T.neq, vp(IAd), vp(JAd), vp(AAd), vp(Pd.data_ptr()), vp(Qd.data_ptr()),
                                       None) == 0
    torch.cuda.synchronize()
    Qf = Qd.cpu().numpy()[:T.neq]
    IA, JA = pat["IA"], pat["JA"]
    rows = np.repeat(np.arange(T.neq), np.diff(IA))
    mag = np.bincount(rows, weights=np.abs(A[:IA[-1]] * P[JA]), minlength=T.neq)
    bound = 2.0 * np.diff(IA) * np.finfo(np.float64).eps * mag
    assert np.all(np.abs(Qf - Qref[:T.neq]) <= bound), "fused CSR product"


def test_transport_c2_structure_build_matvec_ilu0_bitexact(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(2048, 1024, perturb=0.2, seed=1234)
    p = skew_problem(m)
    ref = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc, p.upresc,
                                 scheme="CSR", reord="SYMRCM", precond="ILU0", kmax=50, lmax=1000, tol=1e-8,
                                 npicard=1)
    assert ref["neq"] == 2097152 and ref["nnzero"] == 14667778
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", kmax=50) as T:
        assert T.neq == ref["neq"] and T.nnzero == ref["nnzero"] and T.bandwidth == ref["bandwidth"]
        pat = T.pattern()
        assert np.array_equal(pat["node_id"], ref["node_id"]), "SYMRCM renumbering"
        assert np.array_equal(pat["IA"], ref["IA"]), "IA"
        assert np.array_equal(pat["JA"], ref["JA"]), "JA"
        assert np.array_equal(pat["sbe"], ref["sbe"]), "CSR_by_Element"
        F, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
        assert np.array_equal(A, ref["Afirst"]), "matrix"
        assert np.array_equal(F, ref["Ffirst"]), "RHS"
        Q = T.ProductMatrixVector(ref["Pin"])
        assert np.array_equal(Q, ref["Qmv"]), "csrmv"
        _check_fused_product(T, pat, A, ref["Pin"], ref["Qmv"])
        Fp = T.precond_setup(1)
        assert np.array_equal(Fp, ref["Fprec"]), "F := M^-1 F"
        Z = T.precond(ref["Pin"])
        assert np.array_equal(Z, ref["Zpc"]), "ILU(0) application"


def test_euler_c3_build_bitexact(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(1024, 256, lx=4.0, ly=1.0)
    pb = refletido_problem(m)
    assert m.nel == 524288
    rng = np.random.default_rng(17)
    u = pb.u0 * (1.0 + 0.05 * rng.uniform(-1, 1, pb.neq + 1))
    du = 0.1 * rng.uniform(-1, 1, pb.neq + 1)
    u[pb.neq] = du[pb.neq] = 0.0
    dt = euler_cfl_dt(m, 5.0)
    Ao, Ro = pyoracle.euler_build(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, u, du, alpha=0.5, dt=dt,
                                  stab_tol=1e-6)
    with fg.Euler.from_problem(m, pb, alpha=0.5, dt=dt, stab_tol=1e-6) as eu:
        R, Ae = eu.Build(u, du, want_matrix=True)
    assert np.array_equal(R, Ro), "residual"
    assert np.array_equal(Ae, Ao), "element Jacobians"


def test_euler_predictor_two_steps_256x64_fp64(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(256, 64, lx=4.0, ly=1.0)
    pb = refletido_problem(m)
    dt = euler_cfl_dt(m, 5.0)
    uo, ito = pyoracle.euler_predictor(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, pb.u0, 2, 2, dt=dt,
                                       kmax=50, lmax=100, tol=1e-8)
    with fg.Euler.from_problem(m, pb, dt=dt, kmax=50, lmax=100, tol=1e-8, ncorr=2) as eu:
        uh, its = eu.Predictor(pb.u0, 2)
    assert _rel(uh, uo) < SOL_RTOL, _rel(uh, uo)
    assert np.abs(its.astype(int) - ito.astype(int)).max() <= 1, (its, ito)
