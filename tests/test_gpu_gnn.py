"""Learned preconditioner on the GPU: the CUDA forward pass, hand-written
backward pass and Adam step against the CPU oracle (oracle/gnn_oracle.py),
and a trained network's gain inside FGMRES.

Tolerances: with FP32 activations the GPU and the oracle differ only in the
order of FP32 accumulations (relative 1e-4 on z, 1e-3 on the gradient);
with bf16 activations a rounding flip in a stored activation moves results
by about 2^-8, so the bars are relative 2e-2 (z) and 5e-2 (gradient)."""
import numpy as np
import pytest

from oracle import gnn_oracle as G
from oracle import pyoracle
from fem_codes_gb300.mesh import rotated_problem, structured_mesh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    m = structured_mesh(40, 30, perturb=0.2, seed=3)
    pb = rotated_problem(m, 2.1, 1e-3)
    out = pyoracle.run_transport(m.x, m.y, pb.node_type, m.vert, pb.k, pb.gamma, pb.beta, pb.fsrc, pb.upresc,
                                 npicard=1)
    IA, JA, AA = out["IA"], out["JA"], out["Afirst"]
    rng = np.random.default_rng(4)
    n = out["neq"]
    r = rng.normal(size=n)
    t = pyoracle.ilu0_apply(IA, JA, *pyoracle.ilu0(IA, JA, AA), np.append(r, 0.0))[:n]
    return IA, JA, AA, r, t


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("bf16,ztol,gtol,loss", [(False, 1e-4, 1e-3, "supervised"), (True, 2e-2, 5e-2, "supervised"),
                                                  (False, 1e-4, 1e-3, "residual"), (False, 1e-4, 1e-3, "both")])
def test_forward_backward_vs_oracle(gpu_lib, system, bf16, ztol, gtol, loss):
    from fem_codes_gb300.learned import MeshGNN
    IA, JA, AA, r, t = system
    th = G.init(7)
    g = G.graph(IA, JA, AA)
    Lo, go, zo = G.loss_and_grad(th, g, r, t, act_bf16=bf16, kind=MeshGNN.LOSSES[loss])
    net = MeshGNN(th, bf16=bf16)
    net.set_loss(loss)
    net.attach_csr(IA, JA, AA[: len(JA)])
    z = net.apply(r)
    assert _rel(z, zo) < ztol
    L, gr, z2 = net.loss_grad(r, t)
    assert np.array_equal(z, z2)
    assert abs(L - Lo) / Lo < ztol
    assert _rel(gr, go) < gtol
    net.close()


def test_adam_step_vs_oracle(gpu_lib, system):
    from fem_codes_gb300.learned import MeshGNN
    IA, JA, AA, r, t = system
    th = G.init(3)
    net = MeshGNN(th, bf16=False)
    net.attach_csr(IA, JA, AA[: len(JA)])
    _, gr, _ = net.loss_grad(r, t)
    net.adam(1e-3, 0.5)
    m = np.zeros_like(th)
    v = np.zeros_like(th)
    ref = G.adam(th.copy(), gr * np.float32(0.5), m, v, 1, 1e-3)
    assert np.abs(net.params() - ref).max() < 1e-6
    net.close()


def test_bad_graph_rejected(gpu_lib):
    """A row without a diagonal entry is reported, not used."""
    import fem_codes_gb300 as fg
    from fem_codes_gb300.learned import MeshGNN
    net = MeshGNN()
    IA = np.array([0, 2, 3], np.int32)
    JA = np.array([0, 1, 0], np.int32)          # row 1 has no diagonal
    AA = np.array([2.0, -1.0, -1.0])
    with pytest.raises(fg.FemGpuError) as e:
        net.attach_csr(IA, JA, AA)
    assert e.value.code == -8
    net.close()


def test_trained_network_beats_no_preconditioner(gpu_lib):
    """Train (residual loss) on the solver's own Arnoldi vectors of a few
    transport problems, then solve held-out problems (other angles,
    diffusivities and seeds) to 1e-8: the learned preconditioner needs far
    fewer FGMRES iterations than the method without it, and every solve
    reaches the tolerance on the true residual."""
    from fem_codes_gb300 import learned as Ld
    train_specs = Ld.sample_problems(8, [48, 64], seed=1)
    sets = [Ld.collect_pairs(s, picard_steps=2, kmax=30) for s in train_specs]
    net = Ld.MeshGNN(seed=0)
    hist = Ld.train(net, sets, epochs=4, lr=2e-3, batch=8, seed=0)
    assert hist[-1] < hist[0]
    tests = Ld.sample_problems(3, [64], seed=99)
    for spec in tests:
        none = Ld.evaluate(spec, None, kmax=30, lmax=400, precond="NOT")
        # stall_ratio 1: never hand over to ILU(0), so the gain is the network's
        lrn = Ld.evaluate(spec, net, kmax=30, lmax=400, stall_ratio=1.0)
        assert lrn["converged"] and lrn["rel"] <= 1.0001e-8
        assert not lrn["fell_back"]
        assert lrn["iters"] < 0.7 * none["iters"], (spec, lrn, none)
    for s in sets:
        s.T.close()
    net.close()


def test_learned_falls_back_to_amg_on_stall(gpu_lib):
    """With an AMG context attached, a stalled learned solve continues with
    the AMG V-cycle (built from the current matrix at the switch) and
    converges on the true residual."""
    import fem_codes_gb300 as fg
    from fem_codes_gb300 import learned as Ld
    net = Ld.MeshGNN(seed=123)
    amg = fg.AMG(ncl=3, beta=-1.0, omega=1.0, nr=2)
    out = Ld.evaluate((48, 0.9, 1e-4, 5), net, kmax=30, lmax=400, stall_ratio=1e-3, amg=amg)
    assert out["fell_back"] == 2 and out["converged"]
    amg.close()
    net.close()


def test_learned_falls_back_to_ilu_on_stall(gpu_lib):
    """An untrained (random) network that does not reduce the residual fast
    enough hands the solve to ILU(0), which then converges; the network
    survives the transport contexts it served."""
    from fem_codes_gb300 import learned as Ld
    net = Ld.MeshGNN(seed=123)
    for spec in [(48, 0.9, 1e-4, 5), (56, 2.0, 1e-3, 6)]:
        out = Ld.evaluate(spec, net, kmax=30, lmax=400, stall_ratio=1e-3)
        assert out["fell_back"] and out["converged"]
    net.close()


def test_update_tensor_cores_match_fp32_cores(gpu_lib, system, monkeypatch):
    """bf16 activations: the tensor-core update (mma.sync m16n8k16, weights
    split into two bf16 parts, FP32 accumulation) against the FP32-core
    update of the same network (FEMGPU_GNN_MMA=0).  The two differ only in
    the accumulation order, so a stored bf16 activation can flip by one
    rounding step: z within relative 1e-2 of each other, and both within
    the oracle's bf16 bar."""
    from fem_codes_gb300.learned import MeshGNN
    IA, JA, AA, r, t = system
    th = G.init(7)
    _, _, zo = G.loss_and_grad(th, G.graph(IA, JA, AA), r, t, act_bf16=True, kind=MeshGNN.LOSSES["supervised"])
    zs = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("FEMGPU_GNN_MMA", mode)
        net = MeshGNN(th, bf16=True)
        net.attach_csr(IA, JA, AA[: len(JA)])
        zs[mode] = net.apply(r)
        assert np.array_equal(zs[mode], net.apply(r))
        net.close()
    assert _rel(zs["1"], zs["0"]) < 1e-2
    assert _rel(zs["1"], zo) < 2e-2 and _rel(zs["0"], zo) < 2e-2
