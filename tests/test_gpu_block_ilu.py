"""Block ILU(0) (ilu_blocks = P): ILU(0) of the block-diagonal part of the
CSR matrix over P contiguous row blocks of the numbering, one thread block
per matrix block on the GPU.  The runs are cut at equal spans of the full
factor's dependency levels (FEMGPU_ILU_BLOCK_CUT=depth: the shallowest
deepest run; =rows: equal row counts); the test reads the cut the library
chose, checks it against its own restatement of each rule, and builds the
oracle's block-diagonal matrix from it.  The preconditioner application is
checked bit for bit against the oracle's ILU(0) of the same block-diagonal
matrix (the reference's factorisation and sweeps applied to the matrix with
the inter-block couplings dropped), and FGMRES with it reaches the
true-residual tolerance."""
import numpy as np
import pytest

from blockcut_ref import block_ids, level_counts, level_cut
from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu


def _block_diag(IA, JA, AA, blk):
    n = len(IA) - 1
    rows = np.repeat(np.arange(n), np.diff(IA))
    keep = blk[rows] == blk[JA]
    IAf = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(np.int32)
    return IAf, JA[keep].astype(np.int32), AA[: len(JA)][keep]


@pytest.mark.parametrize("mode", ["levels", "depth", "rows"])
@pytest.mark.parametrize("nx,ny,P", [(48, 32, 7), (96, 64, 16), (64, 64, 1000)])
def test_block_ilu_apply_bitexact(gpu_lib, nx, ny, P, mode, monkeypatch):
    import fem_codes_gb300 as fg
    if mode == "levels":
        monkeypatch.delenv("FEMGPU_ILU_BLOCK_CUT", raising=False)
    else:
        monkeypatch.setenv("FEMGPU_ILU_BLOCK_CUT", mode)
    m = structured_mesh(nx, ny, perturb=0.2, seed=7)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver="GMRES",
                                     ilu_blocks=P) as T:
        F, AA = T.Build(want_matrix=True)
        T.precond_setup(1)
        pat = T.pattern()
        IA, JA = np.asarray(pat["IA"]), np.asarray(pat["JA"])
        first = T.ilu_blocks()
        P = min(P, T.neq)
        assert first.size == P + 1 and first[0] == 0 and first[-1] == T.neq and np.all(np.diff(first) > 0)
        blk = block_ids(first)
        if mode == "rows":
            assert np.array_equal(blk, np.arange(T.neq, dtype=np.int64) * P // T.neq)
        elif mode == "levels":
            assert np.array_equal(first, level_cut(IA, JA, P))
        else:
            # no contiguous cut into P runs has a shallower deepest run
            depth = level_counts(IA, JA, blk).max()
            assert depth <= level_counts(IA, JA, np.arange(T.neq, dtype=np.int64) * P // T.neq).max()
        IAf, JAf, AAf = _block_diag(IA, JA, AA, blk)
        LU, Dinv = pyoracle.ilu0(IAf, JAf, AAf)
        r = np.random.default_rng(3).uniform(-1, 1, T.neq + 1)
        r[T.neq] = 0.0
        zo = pyoracle.ilu0_apply(IAf, JAf, LU, Dinv, r)
        z = T.precond(r)
    assert np.array_equal(z[: T.neq], zo[: T.neq])


def test_block_ilu_fgmres_converges(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(256, 128, perturb=0.2, seed=1234)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver="FGMRES",
                                     kmax=50, lmax=100, tol=1e-8, ilu_blocks=64) as T:
        T.build_dev()
        T.precond_setup_dev(1)
        it = T.solve_dev()
        rel = T.true_residual()
    assert rel <= 1.0001e-8 and it > 0
