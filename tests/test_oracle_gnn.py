"""The CPU oracle of the learned preconditioner: its hand-derived backward
pass against central finite differences of its own forward pass (double
precision), and the bf16 rounding helper."""
import numpy as np
import pytest

from oracle import gnn_oracle as G
from oracle import pyoracle
from fem_codes_gb300.mesh import rotated_problem, structured_mesh


@pytest.fixture(scope="module")
def small_graph():
    m = structured_mesh(12, 10, perturb=0.2, seed=3)
    pb = rotated_problem(m, 0.7, 1e-3)
    out = pyoracle.run_transport(m.x, m.y, pb.node_type, m.vert, pb.k, pb.gamma, pb.beta, pb.fsrc, pb.upresc,
                                 npicard=1)
    return G.graph(out["IA"], out["JA"], out["Afirst"]), out["neq"]


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_backward_matches_finite_differences(small_graph, kind):
    g, n = small_graph
    rng = np.random.default_rng(0)
    r, t = rng.normal(size=n), rng.normal(size=n)
    th = G.init(1).astype(np.float64)
    _, gr, _ = G.loss_and_grad(th, g, r, t, act_bf16=False, dt=np.float64, kind=kind)
    idx = rng.choice(th.size, 60, replace=False)
    e = 1e-6
    for k in idx:
        tp, tm = th.copy(), th.copy()
        tp[k] += e
        tm[k] -= e
        fd = (G.loss_and_grad(tp, g, r, t, act_bf16=False, dt=np.float64, kind=kind)[0] -
              G.loss_and_grad(tm, g, r, t, act_bf16=False, dt=np.float64, kind=kind)[0]) / (2 * e)
        assert abs(fd - gr[k]) <= 1e-6 * max(1.0, abs(gr).max()), k


def test_param_count_and_layout():
    assert G.nparams() == 9441
    th = G.init(0)
    p = G.unpack(th)
    assert p["We"].shape == (2, 32) and p["Wh2"].shape == (32, 32) and p["bd"].shape == (1,)
    assert np.array_equal(G.pack(p), th)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-40], np.float32)
    b = G.bf16(x)
    assert b[0] == 1.0 and b[1] == 1.0            # tie to even
    assert b[2] == np.float32(1.0078125)          # above the tie rounds up
    assert abs(b[3] + 3.140625) < 1e-6
    assert (b.view(np.uint32) & 0xFFFF == 0).all()
