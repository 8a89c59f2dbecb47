"""Training of the learned chain-preconditioner network on reduced camera
systems produced by this bundle adjuster.

Maps are drawn like the 2,000-keyframe benchmark map (same generator recipe:
frustum landmarks, geometric tracks of mean 8 capped at 40, two cameras) with
seeds ``seed0 .. seed0 + maps - 1`` and ``keyframes`` keyframes each.  On every
map the device LM advances one iteration at a time (mixed precision, chain
preconditioner); at each state the network takes ``steps`` Adam steps on that
state's reduced system (probe loss mean |T^-1 S w - w|^2, see
include/maplab_ba.h: mba_gnn_train).  Each (map, iteration) is one training
system.

    python -m maplab_gb300.train_preconditioner --maps 250 --iters 20 \
        --out maplab_gb300/data/chain_precond_gnn.npy
"""
import argparse
import json
import os
import time

import numpy as np

from . import _native as N
from . import ba, synth

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "chain_precond_gnn.npy")


def load_default_model(device=0):
    """The trained model shipped with the package (None if absent)."""
    if not os.path.exists(DEFAULT_WEIGHTS):
        return None
    return ba.PreconditionerModel.load(DEFAULT_WEIGHTS, device=device)


def train(maps=250, iters=20, steps=2, nprobe=4, lr=1e-3, keyframes=500, landmarks_per_kf=100, seed0=1000,
          device=0, model=None, log=print):
    model = model or ba.PreconditionerModel(device=device, seed=seed0)
    history = []
    t0 = time.time()
    for mi in range(maps):
        m = synth.generate("c2", seed=seed0 + mi, keyframes_per_mission=keyframes,
                           num_landmarks=landmarks_per_kf * keyframes)
        with ba.BundleAdjuster(m.desc, device=device) as g:
            radius = 1e5
            map_losses = []
            for it in range(iters):
                try:
                    losses = g.train_preconditioner(model, radius, nprobe=nprobe, steps=steps, lr=lr,
                                                    seed=(seed0 + mi) * 1000 + it)
                    map_losses.append(float(losses[0]))
                except ba.BAError:
                    pass  # system not positive definite under these coefficients: skipped
                o = ba.default_options(max_num_iterations=1, initial_trust_region_radius=radius,
                                       precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN,
                                       max_linear_iterations=25, check_tolerances=0, reject_outliers_every_n_iters=0)
                s = g.solve(o)
                if len(s["iterations"]) > 1:
                    radius = s["iterations"][1]["radius"]
        history.append(float(np.mean(map_losses)) if map_losses else float("nan"))
        if log and (mi % 10 == 0 or mi == maps - 1):
            log(json.dumps({"map": mi, "systems": (mi + 1) * iters, "mean_loss": history[-1],
                            "elapsed_s": round(time.time() - t0, 1)}))
    return model, history


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--maps", type=int, default=250)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--nprobe", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--keyframes", type=int, default=500)
    ap.add_argument("--seed0", type=int, default=1000)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--history", default=None)
    a = ap.parse_args()
    model, hist = train(a.maps, a.iters, a.steps, a.nprobe, a.lr, a.keyframes, seed0=a.seed0)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    model.save(a.out)
    if a.history:
        with open(a.history, "w") as f:
            json.dump({"mean_loss_per_map": hist, "args": vars(a)}, f)
    model.close()


if __name__ == "__main__":
    main()
