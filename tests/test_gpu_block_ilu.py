"""Block ILU(0) (ilu_blocks = P): ILU(0) of the block-diagonal part of the
CSR matrix over P contiguous row blocks of the numbering, one thread block
per matrix block on the GPU.  The preconditioner application is checked
bit for bit against the oracle's ILU(0) of the same block-diagonal matrix
(the reference's factorisation and sweeps applied to the matrix with the
inter-block couplings dropped), and FGMRES with it reaches the true-residual
tolerance."""
import numpy as np
import pytest

from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu


def _block_diag(IA, JA, AA, P):
    n = len(IA) - 1
    rows = np.repeat(np.arange(n), np.diff(IA))
    blk = (np.arange(n, dtype=np.int64) * P // n).astype(np.int64)
    keep = blk[rows] == blk[JA]
    IAf = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=n))]).astype(np.int32)
    return IAf, JA[keep].astype(np.int32), AA[: len(JA)][keep]


@pytest.mark.parametrize("nx,ny,P", [(48, 32, 7), (96, 64, 16), (64, 64, 1000)])
def test_block_ilu_apply_bitexact(gpu_lib, nx, ny, P):
    import fem_codes_gb300 as fg
    m = structured_mesh(nx, ny, perturb=0.2, seed=7)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver="GMRES",
                                     ilu_blocks=P) as T:
        F, AA = T.Build(want_matrix=True)
        T.precond_setup(1)
        pat = T.pattern()
        IAf, JAf, AAf = _block_diag(pat["IA"], pat["JA"], AA, min(P, T.neq))
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
