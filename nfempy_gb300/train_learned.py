"""Train the learned preconditioner's network on the GPU and save it.

    python -m nfempy_gb300.train_learned [--n 16] [--fields 2000] [--out PATH]

Data: plain block-Jacobi FGMRES solves of 3-D mixed Darcy on cube(n) x 6
tetrahedra, one seeded log-normal permeability field per solve (Gaussian
random field, correlation length 0.05, sigma 2.0, seeds 1000 .. 1000+fields),
with the iterate recorded after every restart cycle.  Each solve gives
(residual, error) pairs, turned into per-face flux-extension targets for the
two-level coarse spaces with n/4 and n/8 aggregates per side (learned.py).
Training: Adam with the library's kernels; then alpha (the scale of the
network's correction) is chosen per coarse size on the validation field
(seed 999).  The checkpoint holds the weights, alphas and training record.
"""
import argparse
import json
import os
import time

import numpy as np
import torch

from . import learned

DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "learned_coarse.pt")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--fields", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--out", default=DEFAULT_OUT)
    args = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)
    t0 = time.time()
    P = learned.DarcyProblem(args.n)
    sizes = [max(2, args.n // 8), max(2, args.n // 4)]
    X, T, iters = learned.generate_pairs(P, sizes, range(1000, 1000 + args.fields), log=log)
    t_data = time.time() - t0
    log(f"pairs {tuple(X.shape)} from {len(iters)} solves (plain iterations mean {np.mean(iters):.0f}), {t_data:.0f} s")
    model = learned.MLP(learned.N_FEAT)
    t1 = time.time()
    hist = learned.train(model, X, T, steps=args.steps, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t1
    alphas = {}
    # the aggregate size in cells decides which fraction of the side to use
    for frac in (8, 4):
        nc = max(2, args.n // frac)
        a, res = learned.select_alpha(model, P, nc, seed=999, log=log)
        alphas[frac] = {"alpha": a, "validation_iterations": {str(k): v for k, v in res.items()}}
    ck = {"model": model.state_dict(), "alphas_by_side_fraction": alphas,
          "record": {"n": args.n, "fields": args.fields, "solves_used": len(iters), "pairs": int(X.shape[0]),
                     "plain_iterations_mean": float(np.mean(iters)), "loss_history": hist,
                     "data_seconds": t_data, "train_seconds": t_train}}
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    torch.save(ck, args.out)
    log(json.dumps({"saved": args.out, "alphas": alphas, "train_seconds": t_train}))


def load(path=DEFAULT_OUT, device="cuda"):
    ck = torch.load(path, map_location="cpu", weights_only=True)  # tensors and plain containers only
    model = learned.MLP(learned.N_FEAT, device=device)
    model.load_state_dict(ck["model"])
    return model, ck


if __name__ == "__main__":
    main()
