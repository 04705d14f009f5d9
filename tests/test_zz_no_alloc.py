"""The allocation-free residual-norm entry point (femgpu_csr_resnorm_noalloc)
against the allocating path (femgpu_transport_true_residual) and a numpy FP64
||F - A u||^2 on the same solved system -- two calls in a row, through the C
ABI.  It is meant for host applications that cannot allocate device memory
(a fixed device-memory budget handed to the library, or a driver that must
not grow device memory between steps).  Collected last so that a run
stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu

REL_TOL = 1e-8     # the FP64 parity tolerance of the GPU tests
# ||F - A u|| of a solve converged to 1e-8 cancels about eight digits of F, so
# two FP64 evaluations that round the products differently (fused or not)
# agree in r^2 to ~1e-8 relative, not to 1e-16: compared at 1e-6 relative.
R2_REL_TOL = 1e-6


def test_noalloc_residual_matches_allocating_path(gpu_lib):
    import torch
    import fem_codes_gb300 as fg
    m = structured_mesh(96, 64, perturb=0.2, seed=1234)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", kmax=50,
                                     solver="FGMRES") as T:
        F, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
        T.precond_setup(1)
        u, _ = T.solver()
        expected = T.true_residual()
        pat = T.pattern()
    dev = torch.device("cuda:0")
    IA = torch.from_numpy(pat["IA"]).to(dev)
    JA = torch.from_numpy(pat["JA"]).to(dev)
    AA = torch.from_numpy(A).to(dev)
    ud = torch.from_numpy(u).to(dev)
    Fd = torch.from_numpy(F).to(dev)
    out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    L = gpu_lib
    f = L.femgpu_csr_resnorm_noalloc
    f.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 7
    f.restype = ctypes.c_int
    vp = ctypes.c_void_p
    stream = torch.cuda.current_stream().cuda_stream
    n = len(pat["IA"]) - 1
    # numpy FP64 reference of ||F - A u||^2 and ||F||^2
    import scipy.sparse as sp
    Am = sp.csr_matrix((A[: pat["IA"][-1]], pat["JA"], pat["IA"]), shape=(n, n))
    rr = F[:n] - Am @ u[:n]
    ref_r2 = float(np.dot(rr, rr))
    ref_b2 = float(np.dot(F[:n], F[:n]))
    for call in range(2):
        out.fill_(-1.0)
        rc = f(n, vp(IA.data_ptr()), vp(JA.data_ptr()), vp(AA.data_ptr()), vp(ud.data_ptr()),
               vp(Fd.data_ptr()), vp(out.data_ptr()), vp(stream))
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        r2, b2 = out.cpu().numpy()
        assert abs(b2 - ref_b2) <= REL_TOL * ref_b2, (call, b2, ref_b2)
        assert abs(r2 - ref_r2) <= R2_REL_TOL * ref_r2, (call, r2, ref_r2)
        # the allocating entry point's ||F - A u|| / ||F|| on the same solve
        got = np.sqrt(r2 / b2)
        assert abs(got - expected) <= R2_REL_TOL * expected, (call, got, expected)
        assert got < 1e-7


def test_noalloc_rejects_oversize_and_bad_arguments(gpu_lib):
    f = gpu_lib.femgpu_csr_resnorm_noalloc
    f.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 7
    f.restype = ctypes.c_int
    one = ctypes.c_void_p(1)
    assert f(4 * 1024 * 1024 + 1, one, one, one, one, one, one, None) == -1
    assert f(0, one, one, one, one, one, one, None) == -1
    assert f(10, None, one, one, one, one, one, None) == -1
