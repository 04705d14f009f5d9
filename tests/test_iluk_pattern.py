"""Symbolic ILU(p) on the host (no GPU): the library's level-of-fill pattern
(femgpu_iluk_pattern, the one its ILU(p) contexts factor on) equals the
oracle's restatement of LEVEL_OF_FILL_lu (ilup.c:164-302) row for row, in
the reference's storage order (lower ascending, diagonal, upper in
elimination order), for p = 0..3 on perturbed meshes in both numberings;
p = 0 is the matrix's own pattern; the fill grows with p."""
import numpy as np
import pytest

import fem_codes_gb300 as fg
from oracle import pyoracle
from fem_codes_gb300.mesh import skew_problem, structured_mesh


def _pattern(nx, ny, reord):
    m = structured_mesh(nx, ny, perturb=0.2, seed=4)
    p = skew_problem(m)
    out = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc, p.upresc,
                                 scheme="CSR", reord=reord, precond="NOT", npicard=1)
    return out["IA"], out["JA"]


@pytest.mark.parametrize("reord", ["NOT", "SYMRCM"])
def test_iluk_pattern_matches_oracle(reord):
    IA, JA = _pattern(30, 20, reord)
    prev = None
    for p in range(4):
        fIA, fJA = fg.iluk_pattern(IA, JA, p)
        oIA, oJA = pyoracle.iluk_pattern(IA, JA, p)
        assert np.array_equal(fIA, oIA) and np.array_equal(fJA, oJA), p
        if p == 0:
            assert np.array_equal(fIA, IA)
            for i in range(IA.size - 1):
                assert sorted(fJA[fIA[i]:fIA[i + 1]]) == sorted(JA[IA[i]:IA[i + 1]])
        else:
            assert fIA[-1] > prev
        prev = fIA[-1]
        for i in range(IA.size - 1):                 # lower ascending, then the diagonal
            row = fJA[fIA[i]:fIA[i + 1]]
            lower = row[row < i]
            assert np.all(np.diff(lower) > 0) and row[lower.size] == i


def test_iluk_pattern_rejects_bad_input():
    IA, JA = _pattern(4, 4, "NOT")
    bad = JA.copy()
    bad[0] = IA.size + 5
    with pytest.raises(fg.FemGpuError):
        fg.iluk_pattern(IA, bad, 1)
    with pytest.raises(fg.FemGpuError):
        fg.iluk_pattern(IA, JA, -1)
