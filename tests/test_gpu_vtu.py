"""The VTU output (femgpu_transport_write_vtu) against the file the
reference's Paraview_Output.c writes (tests/golden/vtu_skew16_rcm.npz: the
reference's own final Picard iterate of the 16x16 SYMRCM run, written by the
reference), byte for byte; and the written file of a solved 2048x1024 system
has the reference's structure (one line per node, point and cell)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from fem_codes_gb300.mesh import skew_problem, structured_mesh

pytestmark = pytest.mark.gpu


def test_vtu_bytes_match_reference(gpu_lib, tmp_path):
    import fem_codes_gb300 as fg
    g = dict(np.load(os.path.join(GOLDEN, "vtu_skew16_rcm.npz")))
    m = structured_mesh(16, 16, perturb=0.2, seed=1234)
    p = skew_problem(m)
    assert np.array_equal(m.x, g["x"]) and np.array_equal(m.vert, g["vert"])
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0") as T:
        assert np.array_equal(T.pattern()["node_id"], g["node_id"])
        path = tmp_path / "out.vtu"
        T.write_vtu(str(path), g["u"])
        got = path.read_bytes()
    assert got == bytes(g["vtu"])


def test_vtu_of_a_large_solve(gpu_lib, tmp_path):
    import fem_codes_gb300 as fg
    m = structured_mesh(512, 256, perturb=0.2, seed=1234)
    p = skew_problem(m)
    with fg.SSTransport.from_problem(m, p, scheme="CSR", reorder="SYMRCM", precond="ILU0", solver="FGMRES",
                                     kmax=80, ilu_blocks=8) as T:
        T.build_dev()
        T.precond_setup_dev(1)
        T.solve_dev()
        path = tmp_path / "big.vtu"
        T.write_vtu(str(path))
    lines = path.read_text().splitlines()
    assert lines[2].strip() == f'<Piece NumberOfPoints="{m.nnodes}" NumberOfCells="{m.nel}">'
    assert len(lines) == 2 * m.nnodes + 3 * m.nel + 22
    vals = np.array([float(v) for v in lines[5:5 + m.nnodes]])
    assert np.isfinite(vals).all() and vals.min() > -0.5 and vals.max() < 1.5
