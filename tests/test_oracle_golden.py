"""The CPU oracle (oracle/transport_oracle.c) against the golden vectors that
the reference's own C sources produced (tests/golden/make_golden.py): every
output must be bit-identical.  This pins the oracle before it judges the GPU."""
import numpy as np
import pytest

from conftest import PROBLEM_K_GAMMA, golden_names, load_golden, run_kwargs
from oracle import pyoracle

KEYS_INT = ["neq", "nnzero", "nedge", "bandwidth", "npicard_run", "node_id", "etype", "IA", "JA",
            "sbe", "order", "lm2", "iters"]
KEYS_F64 = ["Afirst", "Ffirst", "Fprec", "Qmv", "Zpc", "uhist"]


@pytest.mark.parametrize("name", golden_names())
def test_oracle_bitexact(name):
    g, meta = load_golden(name)
    k, gamma = PROBLEM_K_GAMMA[meta.get("problem", "SKEW")]
    kw = run_kwargs(meta)
    out = pyoracle.run_transport(g["x"], g["y"], g["node_type"], g["vert"], k, gamma, g["beta"],
                                 g["fsrc"], g["upresc"], Pin=g["Pin"], **kw)
    for key in KEYS_INT + KEYS_F64:
        if key not in g:
            continue
        a, b = np.asarray(out[key]), np.asarray(g[key])
        assert a.shape == b.shape, key
        assert np.array_equal(a, b), f"{name}: {key} differs"


def test_golden_cases_cover_options():
    metas = [load_golden(n)[1] for n in golden_names()]
    assert {m.get("scheme") for m in metas} == {"CSR", "EBE", "EDE"}
    assert {m.get("precond") for m in metas} == {"ILU0", "ILU1", "ILU2", "NOT", "Diag"}
    assert {m.get("shock", "CAU") for m in metas} == {"CAU", "YZBeta"}
    assert {m.get("hshock", "2sqrtArea") for m in metas} == {"2sqrtArea", "sqrtArea", "Option1", "Option2"}
    assert {m.get("reord", "NOT") for m in metas} == {"NOT", "SYMRCM"}


def test_oracle_symrcm_matches_golden_permutation():
    g, meta = load_golden("skew16_csr_ilu0_rcm")
    neq, node_id, lm = pyoracle.fill_lm(g["node_type"], g["vert"])
    IA, JA, _ = pyoracle.csr_pattern(neq, lm)
    perm = pyoracle.symrcm(IA, JA)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(neq)
    mapped = np.where(node_id >= 0, inv[np.maximum(node_id, 0)], -1)
    assert np.array_equal(mapped, g["node_id"])
