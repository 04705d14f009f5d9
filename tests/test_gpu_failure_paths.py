"""Failure paths of the transport context, reached without a GPU fault.

* A zero pivot: an operator that is identically zero (k = 0, gamma = 0,
  beta = 0, zero boundary values) gives the factorisation a zero first pivot;
  the factor kernel records FEMGPU_E_ZERO_PIVOT (the reference prints the
  pivot and exits, CSR/ILUp_precond_setup.c:154-163) and the call returns it.
* A breakdown: a right-hand side with a NaN gives ||b|| = NaN; the solve
  returns FEMGPU_E_BREAKDOWN instead of iterating on NaNs (pgmres.c:85 divides
  by that norm unguarded).
* A wait that runs out: with the sweep warps' dependency-wait bound set to
  zero, every sweep gives up at its first dependent row, records
  FEMGPU_E_TIMEOUT, waits for its copies in flight and returns; the call
  reports the timeout, and after the bound is restored the same context
  applies the preconditioner bit-identically to before and solves to 1e-8.
"""
import numpy as np
import pytest

from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu

E_ZERO_PIVOT, E_BREAKDOWN, E_TIMEOUT = -4, -6, -7


def _transport(fg, solver="FGMRES", ilu_blocks=4, nx=96, ny=64):
    m = structured_mesh(nx, ny, perturb=0.2, seed=5)
    p = skew_problem(m)
    return fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver=solver,
                                       kmax=30, lmax=2000, tol=1e-8, ilu_blocks=ilu_blocks)


def test_zero_pivot_reported(gpu_lib):
    import fem_codes_gb300 as fg
    m = structured_mesh(24, 16, perturb=0.2, seed=2)
    p = skew_problem(m)
    with fg.SSTransport(m.x, m.y, p.node_type, m.vert, 0.0, 0.0, np.zeros(m.nnodes), const_beta=(0.0, 0.0),
                        scheme="CSR", precond="ILU0") as T:
        F, A = T.Build(want_matrix=True)
        assert not np.any(A)
        with pytest.raises(fg.FemGpuError) as e:
            T.precond_setup()
        assert e.value.code == E_ZERO_PIVOT


def test_nan_rhs_breakdown(gpu_lib):
    import fem_codes_gb300 as fg
    with _transport(fg) as T:
        F, _ = T.Build()
        T.precond_setup()
        B = F.copy()
        B[T.neq // 2] = np.nan
        with pytest.raises(fg.FemGpuError) as e:
            T.solver_bx(B)
        assert e.value.code == E_BREAKDOWN
        X, it = T.solver_bx(F)                      # the context is still usable
        assert np.all(np.isfinite(X[:T.neq])) and it > 0


@pytest.mark.parametrize("solver", ["FGMRES", "GMRES"])
def test_sweep_wait_runs_out_then_recovers(gpu_lib, solver):
    """FGMRES runs the chain-scan sweeps (k_sweep_cs), the reference's GMRES
    the row-by-row dataflow sweeps (k_sweep_df): both give up the same way."""
    import fem_codes_gb300 as fg
    with _transport(fg, solver=solver) as T:
        F, _ = T.Build()
        T.precond_setup()
        r = np.random.default_rng(0).standard_normal(T.neq + 1)
        z0 = T.precond(r)
        X0, it0 = T.solver_bx(F)
        T.set_sweep_wait(0)
        with pytest.raises(fg.FemGpuError) as e:
            T.precond(r)
        assert e.value.code == E_TIMEOUT
        with pytest.raises(fg.FemGpuError) as e:
            T.solver_bx(F)
        assert e.value.code == E_TIMEOUT
        T.set_sweep_wait(-1)
        z1 = T.precond(r)
        assert np.array_equal(z0[:T.neq], z1[:T.neq])
        X1, it1 = T.solver_bx(F)                    # the solve starts from zero, as pgmres.c:46
        assert it1 == it0 and np.array_equal(X0[:T.neq], X1[:T.neq])
        if solver == "FGMRES":
            assert T.true_residual() <= 1e-8
