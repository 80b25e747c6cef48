"""Train the learned closure of the coarse 3-D dam break and save it.

    python -m cmag_gb300.train_closure [--seeds 20] [--window 10] [--t-train 1.0]
        [--sample-every 0.025] [--steps 4000] [--time-budget S]
        [--out cmag_gb300/data/closure_dambreak3d.npz]

The fine run is the 64x128x64 dam break (dt 5e-5), the coarse run its 2x-coarser
twin (32x64x32 fluid, dt 1e-4).  For each training seed (jitter seeds 2001, 2002,
...) the two advance in lockstep from the same initial state to t_train; every
sample_every seconds the coarse fluid particles' features are recorded with their
time-filtered targets (closure.collect_filtered: the missed acceleration averaged
over the `window` coarse steps ending at the sample).  The network is trained by
the library's own forward/backward/Adam kernels; the plain fine run then judges
it on a validation seed (998) and fixes the strength of the correction
(closure.choose_strength: 0 falls back to the plain coarse method).  Seeds 998 and
the benchmark's 1973 are never trained on.

The saved file holds the FP32 parameters, the input normalisation, the output
scale and clamp, the chosen strength and the training record; load() rebuilds the
closure from it.
"""
import argparse
import json
import os
import time

import numpy as np

from . import closure as C

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "data", "closure_dambreak3d.npz")
COLUMN_WIDTH = 0.5  # the fine column's width (m): fronts are normalised by it


def save(path, closure, strength, record):
    mean, inv, scale = closure.normalization()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=closure.params, mean=mean, inv_std=inv, out_scale=np.float32(scale),
             strength=np.float32(strength), output_limit=np.float32(record["output_limit"]),
             record=np.array(json.dumps(record)))


def load(path=DEFAULT_OUT):
    """(closure with the saved parameters, normalisation, clamp and the chosen
    strength folded into its output scale, the saved record)."""
    d = np.load(path)
    c = C.Closure(d["params"])
    c.set_normalization(d["mean"], d["inv_std"], float(d["out_scale"]) * float(d["strength"]))
    c.set_output_limit(float(d["output_limit"]))
    record = json.loads(str(d["record"]))
    record["strength"] = float(d["strength"])
    return c, record


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--seeds", type=int, default=20)
    ap.add_argument("--window", type=int, default=10)
    ap.add_argument("--t-train", type=float, default=1.0)
    ap.add_argument("--sample-every", type=float, default=0.025)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--time-budget", type=float, default=None,
                    help="seconds of data collection after which no further seed starts")
    args = ap.parse_args()
    run(args.seeds, args.window, args.t_train, args.sample_every, args.steps, args.out,
        time_budget=args.time_budget)


def initial_params(seed=0):
    """He-style initial parameters for the 16-64-64-64-3 network (weights of a
    layer ~ N(0, 2 / fan_in), biases 0), in the library's order W1 b1 W2 b2 W3 b3
    W4 b4 with W[out][in]; the last layer starts small."""
    rng = np.random.default_rng(seed)
    shapes = [(64, 16), (64, 64), (64, 64), (3, 64)]
    out = []
    for k, (o, i) in enumerate(shapes):
        w = rng.normal(0.0, np.sqrt(2.0 / i), size=(o, i))
        if k == len(shapes) - 1:
            w *= 0.1
        out += [w.ravel(), np.zeros(o)]
    return np.concatenate(out).astype(np.float32)


def run(seeds=20, window=10, t_train=1.0, sample_every=0.025, steps=4000, out=DEFAULT_OUT, valid_seed=998,
        log=print, time_budget=None):
    import torch
    pair = C.Pair()
    fine_dt = float(pair.pf.delta_time)
    every = 2 * int(round(sample_every / (2 * fine_dt)))
    snaps = int(round(t_train / sample_every))
    train_seeds = list(range(2001, 2001 + seeds))
    t0 = time.perf_counter()
    done = []
    feat, tgt = C.collect_filtered(pair, train_seeds, snaps, every, window,
                                   deadline=None if time_budget is None else t0 + time_budget, done=done)
    train_seeds = done
    t_data = time.perf_counter() - t0
    log("data: %d rows from %d seeds in %.1f s" % (feat.shape[0], len(train_seeds), t_data))
    c = C.Closure(initial_params(0))
    mean, inv, scale = C.normalization_from(feat, tgt)
    c.set_normalization(mean, inv, scale)
    limit = C.output_limit_from(tgt, scale)
    c.set_output_limit(limit)
    t0 = time.perf_counter()
    losses = C.train(c, feat, tgt, steps=steps, batch=65536, lr=2e-3, lr_final=1e-4,
                     log_every=max(1, steps // 10))
    torch.cuda.synchronize()
    t_train_s = time.perf_counter() - t0
    log("training: %d Adam steps in %.1f s, losses %s" % (steps, t_train_s, losses))
    rows = int(feat.shape[0])
    del feat, tgt
    t0 = time.perf_counter()
    strength, verr = C.choose_strength(pair, c, valid_seed, 1.0, COLUMN_WIDTH)
    t_valid_s = time.perf_counter() - t0
    log("validation (seed %d): strength %.2f, front errors %s" % (valid_seed, strength, verr))
    # choose_strength folded the strength into the output scale: store the
    # unscaled normalisation and the strength separately
    c.set_normalization(mean, inv, scale)
    record = {"train_seeds": train_seeds, "validation_seed": valid_seed, "window_coarse_steps": window,
              "t_train": t_train, "sample_every": sample_every, "rows": rows, "adam_steps": steps,
              "losses": losses, "validation_front_err": {str(f): list(v) for f, v in verr.items()},
              "data_s": t_data, "train_s": t_train_s, "validation_s": t_valid_s, "output_limit": limit,
              "fine": list(pair.fluid_f), "coarse": list(pair.fluid_c)}
    save(out, c, strength, record)
    pair.close()
    c.close()
    log("saved %s" % out)
    return record


if __name__ == "__main__":
    main()
