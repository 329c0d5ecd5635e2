"""Trains the learned preconditioner on solver-generated pairs and evaluates it.

    python -m gridap_gb300.train_learned --cells 96 --fields 500 --epochs 8 --out learned.gdlp

For each training field (kappa = exp(GRF), distinct seeds) the load is M f with
f ~ N(0,1) per node; the solver produces pairs (r_k, e_k) from its own iterates
(see learned.solver_pairs).  Training runs on the GPU with the library's kernels
(Adam, one field's pairs per step).  Evaluation solves held-out fields with
Jacobi-preconditioned and learned flexible CG (both inside the same FP64
refinement) to 1e-8 relative residual and prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main(argv=None):
    import torch
    import gridap_gb300 as G
    from gridap_gb300.learned import LearnedPreconditioner, solver_pairs
    from gridap_gb300.synthetic import DIFFUSION3D_96, gaussian_random_field_torch, lognormal_kappa

    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=96)
    ap.add_argument("--fields", type=int, default=500)
    ap.add_argument("--ks", default="4,16,64,256")
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--levels", type=int, default=3)
    ap.add_argument("--coarse-start", action="store_true", help="network on the once-restricted lattice")
    ap.add_argument("--eval-fields", type=int, default=3)
    ap.add_argument("--init", default=None, help="start from a saved parameter file")
    ap.add_argument("--out", default="learned.gdlp")
    ap.add_argument("--time-budget", type=float, default=1e9, help="seconds for pair generation + training")
    a = ap.parse_args(argv)
    w = dict(DIFFUSION3D_96)
    cells = (a.cells,) * 3
    ks = tuple(int(k) for k in a.ks.split(","))
    t_start = time.perf_counter()
    be = G.GB300Backend(0)
    ranks = be.distribute(range(8))
    model = G.CartesianDiscreteModel(ranks, w["parts"], w["domain"], cells)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), 2)
    nnodes = (a.cells + 1) ** 3
    rng = np.random.default_rng(w["seed"])

    def field(seed):
        return torch.exp(gaussian_random_field_torch(cells, w["sigma"], w["corr_len"], seed)).cpu().numpy()

    kap0 = field(1)
    f0 = rng.standard_normal(nnodes)
    op = G.AffineFEOperator(G.integral_grad_grad(kap0, dO), G.integral_source(f0, dO), U, V)
    levels, cs = LearnedPreconditioner.file_spec(a.init) if a.init else (a.levels, a.coarse_start)
    net = LearnedPreconditioner(op.matrix, seed=3, levels=levels, coarse_start=cs)
    if a.init:
        net.load(a.init)

    # ---- pairs from the solver ----
    data = []
    t0 = time.perf_counter()
    for s in range(a.fields):
        if time.perf_counter() - t_start > 0.5 * a.time_budget:
            break
        kap = field(10 + s)
        f = rng.standard_normal(nnodes)
        op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(f, dO))
        b = torch.tensor(op.vector.global_values(), device="cuda")
        r, e = solver_pairs(op.matrix, b, ks=ks)
        data.append((kap, r, e))
    t_pairs = time.perf_counter() - t0

    # ---- training ----
    t0 = time.perf_counter()
    hist = []
    order = np.arange(len(data))
    for ep in range(a.epochs):
        rng.shuffle(order)
        ep_loss = []
        for i in order:
            kap, r, e = data[i]
            op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(0.0, dO))
            lr = a.lr * (0.5 ** (ep // max(1, a.epochs // 3)))
            ep_loss.append(net.train_step(r, e, lr=lr))
            if time.perf_counter() - t_start > a.time_budget:
                break
        hist.append(float(np.mean(ep_loss)))
        if time.perf_counter() - t_start > a.time_budget:
            break
    t_train = time.perf_counter() - t0
    net.save(a.out)

    # ---- evaluation on held-out fields (numpy GRF stream, the benchmark's generator) ----
    evals = []
    for s in range(a.eval_fields):
        kap = lognormal_kappa(cells, w["sigma"], w["corr_len"], seed=w["seed"] + 1 + s)
        f = np.random.default_rng(w["seed"] + 100 + s).standard_normal(nnodes)
        op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(f, dO))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xj = op.matrix.solve(rtol=1e-8, method="mixed_ir")
        tj = time.perf_counter() - t0
        itj = op.matrix.last_stats.iterations
        t0 = time.perf_counter()
        xl, st, fb = net.solve(rtol=1e-8)
        tl = time.perf_counter() - t0
        evals.append({"jacobi_s": tj, "jacobi_iters": itj, "learned_s": tl, "learned_iters": st.iterations,
                      "learned_rel_residual": st.rel_residual, "fallback": fb, "speedup": tj / tl,
                      "max_rel_diff": float(np.abs(xl - xj).max() / np.abs(xj).max())})
    print(json.dumps({"levels": levels, "coarse_start": cs, "params": net.num_params, "pairs": sum(len(d[1]) for d in data), "fields": len(data), "t_pairs_s": t_pairs,
                      "t_train_s": t_train, "loss_per_epoch": hist, "eval": evals}), flush=True)
    net.close()
    be.close()


if __name__ == "__main__":
    main()
