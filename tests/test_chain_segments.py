"""The chain-scan segmentation of the ILU(0) sweeps on the host (no GPU):
femgpu_ilu_chain_segments gives the slots that the chain-scan sweep kernel
(k_sweep_cs) runs.  Checked here:

* structure: every row in exactly one slot, levels starting at multiples of
  32, each 32-slot chunk holding whole segments, a chained row sitting in the
  slot after its sweep predecessor, every other dependency on an earlier
  level -- for the global factor and for block cuts;
* arithmetic: the sweeps emulated slot by slot the way the kernel computes
  them (the row's other terms first, then the five Kogge-Stone steps over the
  chunk's 32 lanes with the multipliers of k_chain_mult) reproduce the
  oracle's ILU(0) application to 1e-12 relative;
* depth: on a SYMRCM-ordered transport mesh the segments remove most of the
  dependency levels (the reason the kernel exists)."""
import numpy as np
import pytest

import fem_codes_gb300 as fg
from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh


def _system(nx, ny, reord="SYMRCM"):
    m = structured_mesh(nx, ny, perturb=0.2, seed=1234)
    p = skew_problem(m)
    out = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc, p.upresc,
                                 scheme="CSR", reord=reord, precond="ILU0", npicard=1)
    return out["IA"], out["JA"], out["Afirst"][:-1]


def _check_structure(IA, JA, seg, lower, blocks):
    n = IA.size - 1
    row, pred, lstart = seg["slot_row"], seg["slot_pred"], seg["lstart"]
    assert np.all(lstart % 32 == 0) and lstart[0] == 0 and lstart[-1] == row.size
    real = row[row >= 0]
    assert np.array_equal(np.sort(real), np.arange(n))
    level = np.zeros(n, np.int64)
    slot = np.zeros(n, np.int64)
    for l in range(seg["levels"]):
        for q in range(lstart[l], lstart[l + 1]):
            if row[q] >= 0:
                level[row[q]] = l
                slot[row[q]] = q
    for q in range(row.size):
        r = row[q]
        if r < 0:
            assert pred[q] == -1
            continue
        step = -1 if lower else 1
        if pred[q] >= 0:
            assert q % 32 != 0, "a segment straddles two chunks"
            assert row[q - 1] == r + step and JA[pred[q]] == r + step
        for k in range(IA[r], IA[r + 1]):
            c = JA[k]
            if (c < r if lower else c > r) and blocks[c] == blocks[r] and k != pred[q]:
                assert level[c] < level[r], (r, c)
    return level


def _emulate(IA, JA, LU, Dinv, seg, x, lower, blocks):
    """One sweep as k_sweep_cs computes it (FP64, fused multiply-adds)."""
    row, pred, lstart = seg["slot_row"], seg["slot_pred"], seg["lstart"]
    out = np.full(IA.size - 1, np.nan)
    for l in range(seg["levels"]):
        for c0 in range(lstart[l], lstart[l + 1], 32):
            a = np.zeros(32)
            b = np.zeros(32)
            for t in range(32):
                r = row[c0 + t]
                if r < 0:
                    continue
                acc = x[r]
                for k in range(IA[r], IA[r + 1]):
                    c = JA[k]
                    if (c < r if lower else c > r) and blocks[c] == blocks[r] and k != pred[c0 + t]:
                        acc = acc - out[c] * LU[k]
                if not lower:
                    acc = acc * Dinv[r]
                a[t] = acc
                if pred[c0 + t] >= 0:
                    b[t] = -LU[pred[c0 + t]] if lower else -(Dinv[r] * LU[pred[c0 + t]])
            M = b.copy()
            for k in range(5):
                d = 1 << k
                a_old, M_old = a.copy(), M.copy()
                a[d:] = a_old[d:] + M_old[d:] * a_old[:-d]
                M[d:] = M_old[d:] * M_old[:-d]
            for t in range(32):
                if row[c0 + t] >= 0:
                    out[row[c0 + t]] = a[t]
    assert not np.isnan(out).any(), "a dependency was read before its level"
    return out


@pytest.mark.parametrize("P", [1, 4])
def test_chain_structure(P):
    IA, JA, _ = _system(40, 24)
    n = IA.size - 1
    first = fg.ilu_block_cut(IA, JA, P)
    blocks = np.zeros(n, np.int64)
    for b in range(first.size - 1):
        blocks[first[b]:first[b + 1]] = b
    for lower in (True, False):
        seg = fg.ilu_chain_segments(IA, JA, P, lower)
        _check_structure(IA, JA, seg, lower, blocks)
        assert seg["deepest"] <= seg["levels"]


def test_chain_sweeps_reproduce_ilu0_application():
    IA, JA, AA = _system(40, 24)
    n = IA.size - 1
    LU, Dinv = pyoracle.ilu0(IA, JA, AA)
    blocks = np.zeros(n, np.int64)
    x = np.random.default_rng(3).uniform(-1.0, 1.0, n + 1)
    ref = pyoracle.ilu0_apply(IA, JA, LU, Dinv, x)[:n]
    lo = fg.ilu_chain_segments(IA, JA, 1, True)
    up = fg.ilu_chain_segments(IA, JA, 1, False)
    y = _emulate(IA, JA, LU, Dinv, lo, x[:n], True, blocks)
    z = _emulate(IA, JA, LU, Dinv, up, y, False, blocks)
    assert np.linalg.norm(z - ref) / np.linalg.norm(ref) < 1e-12


def test_chain_segments_remove_most_levels():
    IA, JA, _ = _system(256, 128)
    for P in (1, 8):
        for lower in (True, False):
            seg = fg.ilu_chain_segments(IA, JA, P, lower)
            assert 4 * seg["deepest"] <= 3 * seg["deepest_rows"], (P, lower, seg["deepest"], seg["deepest_rows"])
            assert seg["width"] <= 3


def test_chain_segments_argument_checks():
    IA, JA, _ = _system(6, 4)
    bad = JA.copy()
    bad[0] = -1
    with pytest.raises(fg.FemGpuError):
        fg.ilu_chain_segments(IA, bad, 1, True)
