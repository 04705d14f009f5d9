"""GPU parity of the ILU(0) triangular sweeps (ILUp_precond.c:26-46) in both
program layouts -- fixed-width row records and ELL sub-blocks -- against the
oracle's ILU(0) (ILUp_precond_setup.c:66-167 / ILUp_precond.c:26-46 restated
in oracle/), on systems that reach the sweep's less common paths:

* levels wider than one 512-row sub-block (a 600x600 mesh in its natural
  numbering has levels of up to ~600 rows), so a level spans two staged
  sub-blocks;
* dependencies older than the shared-memory ring, which the sweep reads back
  from global memory; FEMGPU_SWEEP_NEAR lowers the ring's reach when the
  programs are built, so a small system takes that path for most rows;
* both level synchronisations of the record layout: dataflow (warps wait on
  each other's progress flags, the default) and one barrier per level.

Bar: the separately rounded sweeps (pgmres) are bit-identical to the oracle;
the fused row-by-row sweeps are bit-identical across layouts and ring reaches
and within FMA_TOL of the oracle.

The chain-scan programs (k_sweep_cs, which FGMRES and the FP32 sweeps take
when the factor has them) solve chained rows with a warp scan, so they are
checked against the separately rounded sweeps within CHAIN_TOL, on the same
paths: global and block factors, wide levels, the ring's reach lowered so
most dependencies come back from global memory, and in FP32."""
import os

import numpy as np
import pytest

from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu

FMA_TOL = 1e-12    # fused multiply-subtract vs separately rounded sweeps (relative max-norm)
# chain scan (the recurrence along a segment reassociated over log2(32) steps)
# vs separately rounded sweeps, relative max-norm: FP64 values, and
# double-single values (48-bit significands, a few units of 2^-48 per
# operation, the default for the fused FP64 sweeps)
CHAIN_TOL = 1e-11
DS_TOL = 1e-9


def apply_ilu(m, p, reorder, solver, layout=None, near=None, blocks=0, sync=None, chain="0", info=None, ds=None,
              fb=None):
    """Factor and apply the device ILU(0) of the transport system once; the
    layout, ring reach, level synchronisation (dataflow or one barrier per
    level), the chain-scan programs (chain "0": row-by-row only) and their
    double-single values (ds "0": FP64) are fixed when the sweep programs are
    built."""
    import fem_codes_gb300 as fg
    env = {"FEMGPU_SWEEP_LAYOUT": layout, "FEMGPU_SWEEP_NEAR": near, "FEMGPU_SWEEP_SYNC": sync,
           "FEMGPU_SWEEP_CHAIN": chain, "FEMGPU_SWEEP_DS": ds, "FEMGPU_SWEEP_FB": fb}
    saved = {k: os.environ.get(k) for k in env}
    try:
        for k, v in env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = str(v)
        with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder=reorder, precond="ILU0", solver=solver,
                                         kmax=30, ilu_blocks=blocks) as T:
            _, A = T.Build(u=np.zeros(T.neq + 1), want_matrix=True)
            T.precond_setup(1)
            pat = T.pattern()
            x = np.zeros(T.neq + 1)
            x[:-1] = np.random.default_rng(11).standard_normal(T.neq)
            if info is not None:
                info["chain"] = T.ilu_chain()
            return T.precond(x)[:-1], x, pat, A
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def oracle_apply(pat, A, x):
    IA, JA = np.asarray(pat["IA"]), np.asarray(pat["JA"])
    LU, Dinv = pyoracle.ilu0(IA, JA, A)
    n = IA.size - 1
    return pyoracle.ilu0_apply(IA, JA, LU, Dinv, x)[:n]


@pytest.mark.parametrize("layout,sync", [("rec", "dataflow"), ("rec", "barrier"), ("ell", None)])
def test_levels_wider_than_a_sub_block(gpu_lib, layout, sync):
    m = structured_mesh(600, 600, perturb=0.2, seed=1234)
    p = skew_problem(m)
    z, x, pat, A = apply_ilu(m, p, "NOT", "GMRES", layout=layout, sync=sync)
    assert np.array_equal(z, oracle_apply(pat, A, x))
    zf, _, _, _ = apply_ilu(m, p, "NOT", "FGMRES", layout=layout, sync=sync)
    zr, _, _, _ = apply_ilu(m, p, "NOT", "FGMRES", layout="rec" if layout == "ell" else "ell")
    assert np.array_equal(zf, zr)
    assert np.max(np.abs(zf - z)) <= FMA_TOL * np.max(np.abs(z))


@pytest.mark.parametrize("layout,sync", [("rec", "dataflow"), ("rec", "barrier"), ("ell", None)])
@pytest.mark.parametrize("reorder", ["SYMRCM", "NOT"])
def test_dependencies_older_than_the_ring(gpu_lib, layout, sync, reorder):
    m = structured_mesh(60, 40, perturb=0.2, seed=7)
    p = skew_problem(m)
    z, x, pat, A = apply_ilu(m, p, reorder, "GMRES", layout=layout, near=8, sync=sync)
    assert np.array_equal(z, oracle_apply(pat, A, x))
    zf, _, _, _ = apply_ilu(m, p, reorder, "FGMRES", layout=layout, near=8, sync=sync)
    zd, _, _, _ = apply_ilu(m, p, reorder, "FGMRES", layout=layout, sync=sync)
    assert np.array_equal(zf, zd)


@pytest.mark.parametrize("sync", ["dataflow", "barrier"])
@pytest.mark.parametrize("near", [None, 8])
def test_block_ilu_layouts_agree(gpu_lib, near, sync):
    """Block ILU(0) (couplings between the 4 blocks dropped) has no oracle
    counterpart: both layouts, both synchronisations and both ring reaches
    give the same bits."""
    m = structured_mesh(64, 48, perturb=0.2, seed=3)
    p = skew_problem(m)
    ref, _, _, _ = apply_ilu(m, p, "SYMRCM", "FGMRES", layout="ell", blocks=4)
    z, _, _, _ = apply_ilu(m, p, "SYMRCM", "FGMRES", layout="rec", near=near, blocks=4, sync=sync)
    assert np.array_equal(z, ref)
    assert np.all(np.isfinite(z))


FP32_RTOL = 1e-4   # FP32 sweeps (FP32 factor copies) vs FP64 sweeps, relative max-norm, small systems


@pytest.mark.parametrize("blocks", [0, 4])
def test_fp32_sweeps_both_synchronisations(gpu_lib, blocks):
    """The FP32 programs (the MIXED precision's preconditioner) through the
    device entry point: dataflow and barrier synchronisation give the same
    bits, and the result is the FP64 application to FP32 accuracy."""
    import ctypes
    import torch
    import fem_codes_gb300 as fg
    m = structured_mesh(96, 64, perturb=0.2, seed=5)
    p = skew_problem(m)
    got = {}
    for sync in ("dataflow", "barrier"):
        saved = os.environ.get("FEMGPU_SWEEP_SYNC")
        os.environ["FEMGPU_SWEEP_SYNC"] = sync
        try:
            with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0",
                                             solver="FGMRES", ilu_blocks=blocks) as T:
                T.Build(u=np.zeros(T.neq + 1))
                T.precond_setup(1)
                xh = np.zeros(T.neq + 1)
                xh[:-1] = np.random.default_rng(13).standard_normal(T.neq)
                x = torch.from_numpy(xh).cuda()
                z = torch.zeros(T.neq + 1, dtype=torch.float32, device="cuda")
                torch.cuda.synchronize()
                rc = T._L.femgpu_transport_precond32_dev(T.handle, ctypes.c_void_p(x.data_ptr()),
                                                         ctypes.c_void_p(z.data_ptr()))
                assert rc == 0
                torch.cuda.synchronize()
                got[sync] = (z.cpu().numpy()[:-1].astype(np.float64), T.precond(xh)[:-1])
        finally:
            if saved is None:
                os.environ.pop("FEMGPU_SWEEP_SYNC", None)
            else:
                os.environ["FEMGPU_SWEEP_SYNC"] = saved
    z32, z64 = got["dataflow"]
    assert np.array_equal(z32, got["barrier"][0])
    assert np.array_equal(z64, got["barrier"][1])
    assert np.max(np.abs(z32 - z64)) <= FP32_RTOL * np.max(np.abs(z64))


def _rel_max(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("ds", ["0", None])
@pytest.mark.parametrize("reorder,blocks,near", [("SYMRCM", 0, None), ("SYMRCM", 16, None), ("SYMRCM", 4, 8),
                                                 ("NOT", 0, None), ("NOT", 0, 8)])
def test_chain_sweeps_match_row_sweeps(gpu_lib, reorder, blocks, near, ds):
    """Chain-scan FGMRES sweeps (FP64 or double-single values) against the
    separately rounded row-by-row sweeps of the same factor (global or block),
    with the ring's full or lowered reach; the programs are in use
    (femgpu_transport_ilu_chain)."""
    m = structured_mesh(160, 96, perturb=0.2, seed=21)
    p = skew_problem(m)
    z, x, pat, A = apply_ilu(m, p, reorder, "GMRES", blocks=blocks)
    if blocks == 0:
        assert np.array_equal(z, oracle_apply(pat, A, x))
    info = {}
    zc, xc, _, _ = apply_ilu(m, p, reorder, "FGMRES", blocks=blocks, near=near, chain=None, info=info, ds=ds)
    assert np.array_equal(xc, x)
    assert info["chain"] == 1
    tol = CHAIN_TOL if ds == "0" else DS_TOL
    assert _rel_max(zc, z) <= tol, _rel_max(zc, z)


@pytest.mark.parametrize("reorder,blocks,near", [("SYMRCM", 0, None), ("SYMRCM", 16, None), ("SYMRCM", 4, 8),
                                                 ("NOT", 0, 8)])
def test_fused_forward_backward_sweeps(gpu_lib, reorder, blocks, near):
    """The double-single forward and backward sweeps in one launch (each
    thread block keeps its SM from its block's forward sweep to its backward
    sweep) give the two launches' result bit for bit."""
    m = structured_mesh(160, 96, perturb=0.2, seed=21)
    p = skew_problem(m)
    z2, x2, _, _ = apply_ilu(m, p, reorder, "FGMRES", blocks=blocks, near=near, chain=None, fb="0")
    z1, x1, _, _ = apply_ilu(m, p, reorder, "FGMRES", blocks=blocks, near=near, chain=None, fb="1")
    assert np.array_equal(x1, x2)
    assert np.array_equal(z1, z2)


def test_chain_sweeps_wide_levels(gpu_lib):
    """600x600 cells in the natural numbering: segment levels of several
    32-slot chunks, spanning more than one staged sub-block."""
    m = structured_mesh(600, 600, perturb=0.2, seed=1234)
    p = skew_problem(m)
    z, _, _, _ = apply_ilu(m, p, "NOT", "GMRES")
    info = {}
    zc, _, _, _ = apply_ilu(m, p, "NOT", "FGMRES", chain=None, info=info)
    assert info["chain"] == 1
    assert _rel_max(zc, z) <= DS_TOL, _rel_max(zc, z)


@pytest.mark.parametrize("blocks", [0, 8])
def test_chain_fp32_sweeps(gpu_lib, blocks):
    """The FP32 chain-scan programs (the MIXED precision's preconditioner)
    give the FP64 application to FP32 accuracy."""
    import ctypes
    import torch
    import fem_codes_gb300 as fg
    m = structured_mesh(96, 64, perturb=0.2, seed=5)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver="GMRES",
                                     ilu_blocks=blocks) as T:
        T.Build(u=np.zeros(T.neq + 1))
        T.precond_setup(1)
        assert T.ilu_chain() == 1
        xh = np.zeros(T.neq + 1)
        xh[:-1] = np.random.default_rng(13).standard_normal(T.neq)
        z64 = T.precond(xh)[:-1]
        x = torch.from_numpy(xh).cuda()
        z = torch.zeros(T.neq + 1, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = T._L.femgpu_transport_precond32_dev(T.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(z.data_ptr()))
        assert rc == 0
        torch.cuda.synchronize()
        z32 = z.cpu().numpy()[:-1].astype(np.float64)
    assert np.max(np.abs(z32 - z64)) <= FP32_RTOL * np.max(np.abs(z64))
