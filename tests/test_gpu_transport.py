"""GPU parity of the steady-transport path against the reference's golden
vectors (tests/golden) and against the CPU oracle at larger sizes.

Bar: storage patterns, renumbering, element matrices, assembled storage, RHS,
matvecs and the ILU(0)/diagonal preconditioner are bit-identical to the
reference (the device kernels keep its operation order and round every
operation separately); GMRES solutions, whose dot products are reduced in
parallel, agree to REL_TOL relative L2 per Picard iterate, with the same
iteration counts give or take one."""
import numpy as np
import pytest

from conftest import PROBLEM_K_GAMMA, golden_names, load_golden, run_kwargs
from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu

REL_TOL = 1e-8     # FP64 solution parity (relative L2), as the bar for this path


def make(g, meta, **over):
    import fem_codes_gb300 as fg
    k, gamma = PROBLEM_K_GAMMA[meta.get("problem", "SKEW")]
    kw = run_kwargs(meta)
    opts = dict(scheme=kw["scheme"], reorder=kw["reord"], precond=kw["precond"], shock=kw["shock"],
                hshock=kw["hshock"], outflow=kw["outflow"] == "YES", kmax=kw["kmax"],
                lmax=kw["lmax"], tol=kw["tol"])
    opts.update(over)
    return fg.SSTransport(g["x"], g["y"], g["node_type"], g["vert"], k, gamma, g["upresc"],
                          beta=g["beta"], fsrc=g["fsrc"], **opts), kw


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", golden_names())
def test_structure_and_operators_bitexact(gpu_lib, name):
    g, meta = load_golden(name)
    T, kw = make(g, meta)
    with T:
        assert T.neq == int(g["neq"])
        pat = T.pattern()
        assert np.array_equal(pat["node_id"], g["node_id"])
        if kw["scheme"] == "CSR":
            assert T.nnzero == int(g["nnzero"])
            assert T.bandwidth == int(g["bandwidth"])
            assert np.array_equal(pat["IA"], g["IA"])
            assert np.array_equal(pat["JA"], g["JA"])
            assert np.array_equal(pat["sbe"], g["sbe"])
        elif kw["scheme"] == "EDE":
            assert T.nedge == int(g["nedge"])
            assert np.array_equal(pat["lm2"], g["lm2"])
            assert np.array_equal(pat["sbe"], g["sbe"])
            assert np.array_equal(pat["order"], g["order"])
        F, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
        assert np.array_equal(A, np.asarray(g["Afirst"]).reshape(-1)), "matrix storage"
        assert np.array_equal(F, g["Ffirst"]), "RHS"
        Q = T.ProductMatrixVector(g["Pin"])
        assert np.array_equal(Q, g["Qmv"]), "matvec"
        Fp = T.precond_setup(1)
        assert np.array_equal(Fp, g["Fprec"]), "precond_setup"
        Z = T.precond(g["Pin"])
        assert np.array_equal(Z, g["Zpc"]), "precond"


# Free-running Picard sequences longer than this are compared step by step
# (test_c1_every_picard_iterate_from_the_reference_iterate): the SUPG+CAU
# Picard map of the plain-method configuration stagnates without contracting
# (max |du| ~ 0.04, 51 iterations to the cap), so a rounding-level difference
# in one solve grows from step to step -- measured on GB300, the free-running
# GPU sequence leaves 1e-8 of the reference's at the 16th iterate.
FREE_RUN_STEPS = 8


@pytest.mark.parametrize("name", golden_names())
def test_picard_iterates_match_reference(gpu_lib, name):
    g, meta = load_golden(name)
    T, kw = make(g, meta)
    n = min(kw["npicard"], FREE_RUN_STEPS)
    with T:
        uh, its = T.Process(n)
    ref = g["uhist"][:n]
    assert uh.shape == ref.shape
    for i in range(ref.shape[0]):
        assert rel(uh[i, :-1], ref[i, :-1]) < REL_TOL, f"iterate {i}"
    assert np.all(np.abs(its - g["iters"][:n]) <= 1), (its, g["iters"])


def test_c1_every_picard_iterate_from_the_reference_iterate(gpu_lib):
    """The plain-method configuration (64x64 cells, CSR, ILU(0)-GMRES(30) to
    1e-8, 51 Picard iterations to the reference's cap): every iterate of the
    reference's run is reproduced to 1e-8 by one GPU Picard step (Build,
    precond_setup, pgmres) started from the reference's previous iterate, with
    the reference's GMRES count give or take one; the free-running GPU
    sequence stays within 1e-6 of the reference's over all 51 iterations."""
    g, meta = load_golden("c1_skew64_csr_ilu0_51")
    ref, ref_its = g["uhist"], g["iters"]
    assert ref.shape[0] == 51
    T, kw = make(g, meta)
    with T:
        u_prev = np.zeros(T.neq + 1)
        for i in range(ref.shape[0]):
            T.Build(u=u_prev)
            T.precond_setup(i + 1)
            u, it = T.solver()
            assert rel(u[:-1], ref[i, :-1]) < REL_TOL, f"iterate {i}"
            assert abs(it - int(ref_its[i])) <= 1, (i, it, ref_its[i])
            u_prev = ref[i]
    T, kw = make(g, meta)
    with T:
        uh, its = T.Process(51)
    worst = max(rel(uh[i, :-1], ref[i, :-1]) for i in range(51))
    assert worst < 1e-6, worst


@pytest.mark.parametrize("nx,ny,pert,scheme,reorder,precond", [
    (96, 96, 0.2, "CSR", "SYMRCM", "ILU0"),
    (128, 64, 0.2, "CSR", "NOT", "ILU0"),
    (80, 50, 0.1, "EBE", "NOT", "DIAG"),
    (70, 40, 0.1, "EDE", "NOT", "DIAG"),
])
def test_against_oracle_at_scale(gpu_lib, nx, ny, pert, scheme, reorder, precond):
    import fem_codes_gb300 as fg
    m = structured_mesh(nx, ny, perturb=pert, seed=1234)
    p = skew_problem(m)
    opts = dict(scheme=scheme, reorder=reorder, precond=precond, kmax=30, lmax=1000, tol=1e-8)
    ref = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc,
                                 p.upresc, scheme=scheme, reord=reorder,
                                 precond="Diag" if precond == "DIAG" else precond, npicard=2)
    with fg.SSTransport.from_problem(m, p, **opts) as T:
        pat = T.pattern()
        assert np.array_equal(pat["node_id"], ref["node_id"])
        if scheme == "CSR":
            assert np.array_equal(pat["IA"], ref["IA"]) and np.array_equal(pat["JA"], ref["JA"])
            assert np.array_equal(pat["sbe"], ref["sbe"])
        F, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
        assert np.array_equal(A, np.asarray(ref["Afirst"]).reshape(-1))
        assert np.array_equal(F, ref["Ffirst"])
        uh, its = T.Process(2)
        for i in range(2):
            assert rel(uh[i, :-1], ref["uhist"][i, :-1]) < REL_TOL
        assert T.true_residual() < 1e-6


def test_zero_rhs_gives_zero_solution(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(8, 8)
    p = skew_problem(m)
    with fg.SSTransport(m.x, m.y, p.node_type, m.vert, p.k, 0.0, np.zeros(m.nnodes),
                        const_beta=np.array(p.beta[0])) as T:
        T.Build(u=np.zeros(T.neq + 1))
        T.precond_setup(1)
        u, it = T.solver()
        assert it == 0 and np.all(u == 0)


def test_call_order_and_bad_options(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(4, 4)
    p = skew_problem(m)
    with pytest.raises(fg.FemGpuError):
        fg.SSTransport.from_problem(m, p, scheme="EBE", precond="ILU0")   # ILU is CSR-only
    with fg.SSTransport.from_problem(m, p) as T:
        with pytest.raises(fg.FemGpuError) as e:
            T.precond_setup(1)
        assert e.value.code == -9


def test_single_cell_meshes(gpu_lib):
    import fem_codes_gb300 as fg
    for nx, ny in [(1, 1), (2, 1), (1, 3)]:
        m = structured_mesh(nx, ny)
        p = skew_problem(m)
        if (p.node_type >= 1).sum() == 0:
            continue
        ref = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc,
                                     p.upresc, npicard=1)
        with fg.SSTransport.from_problem(m, p) as T:
            uh, its = T.Process(1)
            assert rel(uh[0, :-1], ref["uhist"][0, :-1]) < REL_TOL
