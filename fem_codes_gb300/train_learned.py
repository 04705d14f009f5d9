"""Train and evaluate the learned preconditioner on transport problems.

    python -m fem_codes_gb300.train_learned [--out PATH] [--problems 20]
        [--sizes 256,512,1024] [--epochs 6] [--eval 4] [--eval-sizes 256,512,1024]

Training set: `--problems` transport problems, mesh size drawn from
`--sizes` (n x n cells, perturbed +-0.2h), velocity angle U[0, 2pi),
diffusivity log-uniform in [1e-6, 1e-2]; from each, the Arnoldi vectors and
ILU(0) corrections of the first FGMRES(50) restart cycle of two Picard steps
(100 pairs per problem: 2000 pairs for 20 problems).  Training runs on the
GPU through the library's own forward/backward kernels and Adam.  The held-
out evaluation solves `--eval` new problems (other seeds) to 1e-8 with
FGMRES(50) and prints one JSON line per problem with the iterations and
seconds of: no preconditioner, ILU(0), and the learned network.  The
parameters are written with numpy.save to --out.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import learned as Ld

DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "gnn_transport.npy")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--problems", type=int, default=20)
    ap.add_argument("--sizes", default="256,512,1024")
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--loss", default="residual")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--eval", type=int, default=4)
    ap.add_argument("--eval-sizes", default="256,512,1024")
    a = ap.parse_args(argv)
    import torch
    torch.cuda.init()
    sizes = [int(s) for s in a.sizes.split(",")]
    t0 = time.perf_counter()
    specs = Ld.sample_problems(a.problems, sizes, seed=a.seed)
    sets = [Ld.collect_pairs(s, picard_steps=2, kmax=50) for s in specs]
    npairs = sum(s.count for s in sets)
    t1 = time.perf_counter()
    net = Ld.MeshGNN(seed=a.seed)
    hist = Ld.train(net, sets, epochs=a.epochs, lr=a.lr, batch=8, seed=a.seed, loss=a.loss)
    t2 = time.perf_counter()
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    np.save(a.out, net.params())
    print(json.dumps({"pairs": npairs, "problems": a.problems, "sizes": sizes, "epochs": a.epochs,
                      "loss": a.loss, "loss_history": [round(h, 4) for h in hist],
                      "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2), "out": a.out}), flush=True)
    for s in sets:
        s.T.close()
    esizes = [int(s) for s in a.eval_sizes.split(",")]
    for spec in Ld.sample_problems(a.eval, esizes, seed=a.seed + 1000):
        row = {"n": spec[0], "angle": round(spec[1], 4), "k": spec[2], "seed": spec[3]}
        for name, gnn, pc, lmax in (("none", None, "NOT", 100), ("ilu0", None, "ILU0", 400),
                                    ("learned", net, None, 400)):
            o = Ld.evaluate(spec, gnn, kmax=50, lmax=lmax, precond=pc, stall_ratio=1.0)
            row[name] = {"iters": o["iters"], "ms": round(1e3 * o["seconds"], 2), "rel": o["rel"]}
        print(json.dumps(row), flush=True)
    net.close()


if __name__ == "__main__":
    main()
