"""The VTU format on the CPU: a restatement of Paraview_Output.c's text
(01_SS_Transport_Equation/2D/01_CommonFiles/Paraview_Output.c:20-83) from
the golden's inputs reproduces the file the reference wrote, byte for byte --
so the golden pins the format the GPU writer must produce
(tests/test_gpu_vtu.py)."""
import os

import numpy as np

from conftest import GOLDEN


def restated_vtu(x, y, vert, node_id, u, upresc):
    nn, ne = len(x), len(vert)
    val = np.where(node_id >= 0, u[np.maximum(node_id, 0)], upresc)
    out = ['<VTKFile type="UnstructuredGrid" version="0.1" byte_order="BigEndian">\n', "\t<UnstructuredGrid>\n",
           f'\t\t<Piece NumberOfPoints="{nn}" NumberOfCells="{ne}">\n', '\t\t\t<PointData Scalars="scalars">\n',
           '\t\t\t\t<DataArray type="Float32" Name="solucao" Format="ascii">\n']
    out += ["\t\t\t\t   %.12f\n" % v for v in val]
    out += ["\t\t\t\t</DataArray>\n", "\t\t\t</PointData>\n", "\t\t\t<Points>\n",
            '\t\t\t\t<DataArray type="Float32" NumberOfComponents="3" Format="ascii">\n']
    out += ["\t\t\t\t   %.12f\t%.12f\t%.12f\n" % (a, b, v) for a, b, v in zip(x, y, val)]
    out += ["\t\t\t\t</DataArray>\n", "\t\t\t</Points>\n", "\t\t\t<Cells>\n",
            '\t\t\t\t<DataArray type="Int32" Name="connectivity" Format="ascii">\n']
    out += ["\t\t\t\t   %d\t%d\t%d\n" % tuple(e) for e in vert]
    out += ["\t\t\t\t</DataArray>\n", '\t\t\t\t<DataArray type="Int32" Name="offsets" Format="ascii">\n']
    out += ["\t\t\t\t   %d\n" % (3 * (i + 1)) for i in range(ne)]
    out += ["\t\t\t\t</DataArray>\n", '\t\t\t\t<DataArray type="Int32" Name="types" Format="ascii">\n']
    out += ["\t\t\t\t   5\n"] * ne
    out += ["\t\t\t\t</DataArray>\n", "\t\t\t</Cells>\n", "\t\t</Piece>\n", "\t</UnstructuredGrid>\n", "</VTKFile>\n"]
    return "".join(out).encode()


def test_restated_vtu_matches_reference_file():
    g = dict(np.load(os.path.join(GOLDEN, "vtu_skew16_rcm.npz")))
    upresc = np.where((g["x"] == 0.0) & (g["y"] > 0.3), 1.0, 0.0)
    got = restated_vtu(g["x"], g["y"], g["vert"], g["node_id"], g["u"], upresc)
    assert got == bytes(g["vtu"])
