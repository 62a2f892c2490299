"""Demo driver (the role of the reference's make_demo2 / load_sim programs): builds a seeded
tissue block, uploads it and runs steps on the GPU.

    python -m morphogenesis_gb300.run --dims 128 64 128 --steps 10 [--param R|L] [--flags 3]
        [--save-state FILE.npz] [--load-state FILE.npz]

Prints particle counts, the run's wall time and, with --profile, per-kernel device times.
--save-state writes every buffer the block uploads (reference layouts) after the run, and
--load-state starts from such a file instead of the fresh block (a checkpoint and restart).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import FluidSystem
from . import _abi as A
from . import demo


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[16, 16, 16])
    ap.add_argument("--param", default="R", choices=["R", "L"])
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--flags", type=int, default=A.STEP_DEFAULT)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--breakable", action="store_true")
    ap.add_argument("--profile", action="store_true")
    ap.add_argument("--tuning", type=int, nargs=4, default=None, metavar=("WARPS", "GROUP", "SUB", "SEARCH"),
                    help="density-pass launch shape (mg_set_tuning)")
    ap.add_argument("--surrogate-train", type=int, default=0,
                    help="train a reaction surrogate for this many Adam steps on pairs captured "
                         "from the block and run the steps with it")
    ap.add_argument("--save-state", default=None)
    ap.add_argument("--load-state", default=None)
    a = ap.parse_args(argv)
    d = demo.make_block(tuple(a.dims), a.param, seed=a.seed, breakable=a.breakable)
    fs = FluidSystem(d.params, d.genome, d.n)
    if a.load_state:
        z = np.load(a.load_state)
        fs.TransferToCL({int(k): z[k] for k in z.files})
    else:
        fs.TransferToCL(d.arrays)
    if a.tuning:
        fs.set_tuning(*a.tuning)
    if a.surrogate_train:
        from . import surrogate as S
        ds = S.Dataset(2 * d.n)
        ds.capture(fs, A.STEP_PHYSICS)
        fs.Run(20)
        ds.capture(fs, A.STEP_PHYSICS)
        mlp = S.Mlp(seed=a.seed)
        mlp.fit_normalization(ds)
        mlp.train(ds, a.surrogate_train, batch=65536)
        ds.close()
        S.attach(fs, mlp, judge_period=10, judge_stride=64, threshold=1e-3)
        a.flags |= A.STEP_SURROGATE
    if a.warmup:
        fs.Run(a.warmup, a.flags)
    if a.profile:
        fs.profile(True)
    t0 = time.perf_counter()
    fs.Run(a.steps, a.flags)
    dt = time.perf_counter() - t0
    out = {"particles": d.n, "steps": a.steps, "seconds": dt, "counts": fs.counts(),
           "particle_steps_per_s": d.n * a.steps / dt}
    if a.profile:
        out["kernels"] = {k: {"launches": v[0], "ms": v[1]} for k, v in fs.profile_read().items()}
    if a.save_state:
        np.savez(a.save_state, **{str(b): fs.download(b) for b in d.arrays})
    print(json.dumps(out))
    fs.close()


if __name__ == "__main__":
    main()
