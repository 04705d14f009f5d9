"""GPU parity of the double-pairwise AMG preconditioner (csrc/amg.cu V-cycle,
host/amg.c set-up) against the reference's own AMG (tests/golden/amg_*.npz,
from amg_precond.c + CSR/AMG/*) and against the CPU oracle's V-cycle at
sizes the fixtures do not reach.

Bar: the hierarchy (every level's CSR and matching), M^-1 F and every
V-cycle are bit-identical to the reference's (level-scheduled SOR that keeps
the sequential sweep's reads, CSR-order sums, no FMA contraction).  The
AMG-preconditioned GMRES, whose dot products are reduced in parallel, takes
the reference's iteration count and agrees to REL_TOL relative L2."""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, PROBLEM_K_GAMMA
from oracle import pyoracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-8
NAMES = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "amg_*.npz")))


def load(name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    L = int(g["nlev"])
    levels = [(g[f"IA{l}"], g[f"JA{l}"], g[f"AA{l}"], g.get(f"rm{l}")) for l in range(L)]
    return g, levels, str(g["spec"])


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_hierarchy_and_vcycle_bitexact(gpu_lib, name):
    import fem_codes_gb300 as fg
    g, levels, spec = load(name)
    amg = fg.AMG.from_spec(spec)
    amg.setup(g["IA"], g["JA"], g["AA"])
    assert amg.levels() == len(levels)
    for l, (IA, JA, AA, rm) in enumerate(levels):
        a, b, c, m = amg.level(l)
        assert np.array_equal(a, IA) and np.array_equal(b, JA), f"level {l} pattern"
        assert np.array_equal(c, AA), f"level {l} values"
        if rm is not None:
            assert np.array_equal(m, rm), f"level {l} matching"
    assert np.array_equal(amg.apply(g["F"]), g["Fprec"]), "F := M^-1 F"
    for k in range(2):
        assert np.array_equal(amg.apply(g["q"][k]), g["z"][k]), f"V-cycle {k}"
    amg.close()


def test_apply_in_place(gpu_lib):
    import torch
    import fem_codes_gb300 as fg
    g, levels, spec = load(NAMES[0])
    amg = fg.AMG.from_spec(spec)
    amg.setup(g["IA"], g["JA"], g["AA"])
    v = torch.tensor(g["q"][1], dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    amg.apply_dev(v.data_ptr(), v.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(v.cpu().numpy(), g["z"][1])
    amg.close()


def _levels_of(amg):
    return [amg.level(l) for l in range(amg.levels())]


@pytest.mark.parametrize("spec", ["AMG 2 3 -1 1.0 2", "AMG 2 2 0.25 0.8 1"])
def test_vcycle_vs_oracle_transport_96x64(gpu_lib, spec):
    """A 6k-row transport matrix (SYMRCM numbering): device V-cycle against
    the oracle's sequential V-cycle over the same hierarchy."""
    import fem_codes_gb300 as fg
    from fem_codes_gb300.mesh import skew_problem, structured_mesh
    mesh = structured_mesh(96, 64, perturb=0.15, seed=3)
    pb = skew_problem(mesh, 1e-3)
    with fg.SSTransport.from_problem(mesh, pb, scheme="CSR", reorder="SYMRCM", precond="NOT") as T:
        F, A = T.Build(want_matrix=True)
        pat = T.pattern()
    IA, JA, AA = pat["IA"], pat["JA"], A[: pat["JA"].size]
    amg = fg.AMG.from_spec(spec)
    amg.setup(IA, JA, AA)
    lv = _levels_of(amg)
    w = spec.split()
    rng = np.random.default_rng(11)
    for _ in range(2):
        q = rng.normal(size=IA.size - 1)
        assert np.array_equal(amg.apply(q), pyoracle.amg_vcycle(lv, float(w[4]), int(w[5]), q))
    amg.close()


def test_vcycle_wide_levels(gpu_lib):
    """A 40k-row matrix whose SOR schedules have levels wider than one thread
    block's run (grid launches per level) mixed with narrow runs."""
    import fem_codes_gb300 as fg
    n, h = 40000, 20000
    rows = [[] for _ in range(n)]
    rng = np.random.default_rng(4)
    for i in range(n):
        rows[i].append((i, 4.0 + rng.uniform()))
    for i in range(h):                       # i <-> i + h: two wide levels
        a, b = -rng.uniform(0.5, 1.0), -rng.uniform(0.5, 1.0)
        rows[i].append((i + h, a))
        rows[i + h].append((i, b))
    for i in range(h, h + 600):              # a chain: narrow levels after them
        rows[i].append((i + 1, -0.3))
        rows[i + 1].append((i, -0.2))
    IA = np.zeros(n + 1, np.int32)
    JA, AA = [], []
    for i in range(n):
        r = sorted(rows[i])
        JA += [c for c, _ in r]
        AA += [v for _, v in r]
        IA[i + 1] = len(JA)
    JA, AA = np.array(JA, np.int32), np.array(AA)
    for spec in ("AMG 2 1 -1 1.1 2", "AMG 2 2 0.1 1.0 1"):
        amg = fg.AMG.from_spec(spec)
        amg.setup(IA, JA, AA)
        lv = _levels_of(amg)
        w = spec.split()
        q = rng.normal(size=n)
        assert np.array_equal(amg.apply(q), pyoracle.amg_vcycle(lv, float(w[4]), int(w[5]), q)), spec
        amg.close()


def _transport(g, **opts):
    import fem_codes_gb300 as fg
    k, gamma = PROBLEM_K_GAMMA[str(g["problem"])]
    return fg.SSTransport(g["x"], g["y"], g["node_type"], g["vert"], k, gamma, g["upresc"], beta=g["beta"],
                          fsrc=g["fsrc"], scheme="CSR", reorder=str(g["reord"]), **opts)


@pytest.mark.parametrize("name", NAMES)
def test_transport_pgmres_amg_vs_reference(gpu_lib, name):
    """FEMGPU_PREC_AMG in the transport context: Build, precond_setup
    (hierarchy + F := M^-1 F) and the left-preconditioned pgmres."""
    import fem_codes_gb300 as fg
    g, levels, spec = load(name)
    with _transport(g, precond="AMG", kmax=int(g["kmax"]), lmax=int(g["lmax"]), tol=float(g["tol"])) as T:
        amg = fg.AMG.from_spec(spec)
        T.set_amg(amg)
        F, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
        assert np.array_equal(A[: g["AA"].size], g["AA"]) and np.array_equal(F[: T.neq], g["F"])
        Fp = T.precond_setup(1)
        assert np.array_equal(Fp[: T.neq], g["Fprec"])
        X, it = T.solver()
        assert abs(it - int(g["iters"])) <= 1
        assert rel(X[: T.neq], g["X"]) < REL_TOL
    amg.close()


def test_transport_fgmres_amg_true_residual(gpu_lib):
    """Right-preconditioned FGMRES with the AMG V-cycle reaches the 1e-8
    true-residual criterion on a 128x96 transport problem."""
    import fem_codes_gb300 as fg
    from fem_codes_gb300.mesh import skew_problem, structured_mesh
    mesh = structured_mesh(128, 96, perturb=0.1, seed=8)
    pb = skew_problem(mesh, 1e-3)
    with fg.SSTransport.from_problem(mesh, pb, scheme="CSR", reorder="SYMRCM", precond="AMG", solver="FGMRES",
                                     kmax=50, lmax=200, tol=1e-8) as T:
        amg = fg.AMG(ncl=3, beta=-1.0, omega=1.0, nr=2)
        T.set_amg(amg)
        T.Build()
        T.precond_setup(1)
        X, it = T.solver()
        assert T.true_residual() <= 1.0000001e-8
        assert it > 0
    amg.close()


def test_transport_amg_requires_context(gpu_lib):
    import fem_codes_gb300 as fg
    g, levels, spec = load(NAMES[0])
    with _transport(g, precond="AMG") as T:
        T.Build()
        with pytest.raises(fg.FemGpuError):
            T.precond_setup(1)
