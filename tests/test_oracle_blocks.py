"""The block (multi-dof) EBE operators of the oracle against the reference's
own ebemvNDOF4/ebe2mvNDOF4/BlockDiag* (Euler) and ebemvNDOF3/BlockDiagDOF3*
(Navier-Stokes) run on the same inputs (tests/golden/blk_*.npz): bit-identical."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import pyoracle

CASES = ["blk_euler_10x6", "blk_ns_9x7"]


def load(name):
    return dict(np.load(f"{GOLDEN}/{name}.npz"))


@pytest.mark.parametrize("name", CASES)
def test_block_oracle_bitexact(name):
    g = load(name)
    ndof, neq = int(g["ndof"]), int(g["neq"])
    out = pyoracle.block_ops(ndof, len(g["x"]), g["vert"], g["node_id"], neq, g["A"], g["P"], g["p"], g["F0"])
    for key in ["Q", "BD", "invBD", "F", "Z"] + (["Q2", "Q2no"] if ndof == 4 else []):
        assert np.array_equal(out[key], g[key]), f"{name}: {key}"
