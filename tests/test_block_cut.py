"""Block ILU(0) cuts on the host (no GPU): femgpu_ilu_block_cut computes the
runs a transport context with ilu_blocks = P uses, on the SYMRCM-numbered
pattern of structured meshes, checked against the Python restatements in
blockcut_ref (the default cut at equal spans of the factor's levels, equal
row counts) and, for the shallowest-run cut, against its defining property."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from blockcut_ref import block_ids, level_counts, level_cut, rows_cut
from fem_codes_gb300.mesh import skew_problem, structured_mesh


def symrcm_pattern(nx, ny):
    """CSR pattern (ascending columns) of the transport unknowns of a
    structured mesh in the library's SYMRCM numbering."""
    import fem_codes_gb300 as fg
    m = structured_mesh(nx, ny, perturb=0.2, seed=11)
    p = skew_problem(m)
    free = np.nonzero(p.node_type >= 1)[0]
    eq = -np.ones(m.nnodes, np.int64)
    eq[free] = np.arange(free.size)
    r = np.repeat(m.vert, 3, axis=1).ravel()
    c = np.tile(m.vert, (1, 3)).ravel()
    k = (eq[r] >= 0) & (eq[c] >= 0)
    n = free.size
    G = sp.csr_matrix((np.ones(int(k.sum())), (eq[r[k]], eq[c[k]])), shape=(n, n))
    G.sum_duplicates()
    G.sort_indices()
    IA, JA = G.indptr.astype(np.int32), G.indices.astype(np.int32)
    perm = np.zeros(n, np.int32)
    L = fg.load()
    L.femgpu_symrcm.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert L.femgpu_symrcm(n, IA.ctypes.data, JA.ctypes.data, perm.ctypes.data) == 0
    Gp = G[perm][:, perm].tocsr()
    Gp.sort_indices()
    return Gp.indptr.astype(np.int32), Gp.indices.astype(np.int32)


@pytest.fixture(scope="module")
def pattern():
    return symrcm_pattern(48, 24)


@pytest.mark.parametrize("P", [2, 7, 16])
def test_default_cut_is_equal_level_spans(pattern, P, monkeypatch):
    import fem_codes_gb300 as fg
    monkeypatch.delenv("FEMGPU_ILU_BLOCK_CUT", raising=False)
    IA, JA = pattern
    assert np.array_equal(fg.ilu_block_cut(IA, JA, P), level_cut(IA, JA, P))


@pytest.mark.parametrize("P", [2, 7, 16])
def test_rows_cut(pattern, P, monkeypatch):
    import fem_codes_gb300 as fg
    monkeypatch.setenv("FEMGPU_ILU_BLOCK_CUT", "rows")
    IA, JA = pattern
    assert np.array_equal(fg.ilu_block_cut(IA, JA, P), rows_cut(IA.size - 1, P))


@pytest.mark.parametrize("P", [2, 7, 16])
def test_depth_cut_is_no_deeper_than_the_others(pattern, P, monkeypatch):
    import fem_codes_gb300 as fg
    monkeypatch.setenv("FEMGPU_ILU_BLOCK_CUT", "depth")
    IA, JA = pattern
    n = IA.size - 1
    first = fg.ilu_block_cut(IA, JA, P)
    assert first.size == P + 1 and first[0] == 0 and first[-1] == n and np.all(np.diff(first) > 0)
    deepest = level_counts(IA, JA, block_ids(first)).max()
    for other in (rows_cut(n, P), level_cut(IA, JA, P)):
        assert deepest <= level_counts(IA, JA, block_ids(other)).max()


def test_degenerate_block_counts(pattern):
    import fem_codes_gb300 as fg
    IA, JA = pattern
    n = IA.size - 1
    assert list(fg.ilu_block_cut(IA, JA, 0)) == [0, n]
    assert list(fg.ilu_block_cut(IA, JA, 1)) == [0, n]
    first = fg.ilu_block_cut(IA, JA, 10 * n)
    assert first.size == n + 1 and np.array_equal(first, np.arange(n + 1))
