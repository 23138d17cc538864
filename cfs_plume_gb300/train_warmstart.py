"""Train the learned pressure warm start (or the preconditioner stage) and
measure what it saves.

    python -m cfs_plume_gb300.train_warmstart --plumes 100 --steps 200 --epochs 4 \
        --out cfs_plume_gb300/weights/unet_warmstart.bin

1. Pairs: `--plumes` randomised closed-box plumes on a 64x96x64 grid (box
   source centre uniform in the middle third of the floor, buoyancy U[0.5, 2],
   vorticity U[0, 4], +-0.05 seeded noise) are simulated with plain MIC-PCG
   (FP32 fields, rel-L2 1e-6); every solve after `--skip` steps is kept on the
   GPU as (b / rms(b), p / rms(b)), or with `--pairs correction` (the default)
   as (r0 / rms(r0), (p - p_prev) / rms(r0)), r0 = b - A p_prev, p_prev the
   previous step's pressure, or with `--pairs iterate` as (r_k / rms(r_k),
   (p - x_k) / rms(r_k)), x_k the iterate after k (1 to 32, below half the
   solve's count) MIC-PCG iterations of the same solve: residuals met
   mid-solve mapped to their errors, the
   preconditioner stage's role.
2. Training: Adam on the network's own BF16 tensor-core forward and backward
   kernels, cosine step size, the last `--val-plumes` plumes held out; the
   loss is the energy norm e^T A e of the error (the norm CG's error bound
   starts from) unless `--loss mse`.
3. Evaluation: the same plume stepped with the zero and the learned initial
   guess at each `--eval-res` (with `--pairs iterate`: plain MIC-PCG against
   flexible CG with the network as the preconditioner), reporting PCG
   iterations per step, steps/s and the relative L2 difference of the final
   velocity.

Everything runs on the GPU; the script only sequences the C ABI calls.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import _abi
from .net import LOSS_ENERGY, LOSS_MSE, PAIRS_CORRECTION, PAIRS_ITERATE, PAIRS_SOLVE, PairStore, PlumeNet
from .plume import Plume


def evaluate(net, res, steps, seed=0, precondition=False):
    """(plain, learned) dicts: iterations per step, ms per step, fallbacks,
    and the final velocity's relative L2 difference.  `precondition`: the
    learned arm uses the network as the flexible-CG preconditioner stage
    (previous-pressure start) instead of as the warm start."""
    out = {}
    vel = {}
    for name, warm in (("plain", _abi.WARM_ZERO), ("learned", _abi.WARM_LEARNED)):
        kw = dict(warm_start=warm)
        if name == "learned" and precondition:
            kw = dict(warm_start=_abi.WARM_PREVIOUS, preconditioner=_abi.PRECOND_NET)
        h = Plume(_abi.plume_config(res, seed=seed, **kw))
        if name == "learned":
            net.attach(h)
        h.run_timed(0, 3)  # warm-up
        ms, stats = h.run_timed(3, steps)
        out[name] = {"iters_per_step": float(np.mean([s.iterations for s in stats])),
                     "ms_per_step": ms / steps,
                     "steps_per_s": 1000.0 * steps / ms,
                     "fallbacks": int(sum(s.fallback for s in stats)),
                     "max_rel_residual": float(max(s.rel_residual for s in stats))}
        vel[name] = h.field("velocity")
        h.close()
    d = np.linalg.norm(vel["learned"] - vel["plain"]) / max(np.linalg.norm(vel["plain"]), 1e-300)
    out["velocity_rel_l2"] = float(d)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", default="64,96,64")
    ap.add_argument("--plumes", type=int, default=100)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--skip", type=int, default=0)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--val-plumes", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=4, help="0: only evaluate --init")
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=5e-5)
    ap.add_argument("--loss", default="energy", choices=["energy", "mse"],
                    help="energy: e^T A e of the error (CG's error norm); mse: squared error")
    ap.add_argument("--pairs", default="correction", choices=["correction", "solve", "iterate"],
                    help="correction: (b - A p_prev) -> p - p_prev; solve: b -> p")
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--out", default=None)
    ap.add_argument("--eval-res", default="64,96,64;128,192,128")
    ap.add_argument("--eval-steps", type=int, default=20)
    ap.add_argument("--log", default=None, help="write the summary JSON here too")
    a = ap.parse_args(argv)
    res = tuple(int(v) for v in a.res.split(","))

    t0 = time.time()
    if a.epochs == 0:  # evaluate given weights only
        if not a.init:
            ap.error("--epochs 0 needs --init")
        net = PlumeNet(path=a.init)
        summary = {"weights": a.init, "eval": {}}
        return finish(a, net, summary, t0)
    ds = PairStore(res, a.plumes, a.steps, skip=a.skip, threads=a.threads, seed=a.seed,
                   kind={"correction": PAIRS_CORRECTION, "solve": PAIRS_SOLVE, "iterate": PAIRS_ITERATE}[a.pairs])
    print("pairs %d from %d plumes in %.1f s (solution rms %.4g)" % (ds.pairs, a.plumes, ds.seconds,
                                                                      ds.target_rms), flush=True)
    net = PlumeNet(seed=a.seed, path=a.init)
    val = a.val_plumes * (a.steps - a.skip)
    tl, vl, secs = net.train(ds, epochs=a.epochs, batch=a.batch, val_pairs=val, lr=a.lr,
                             lr_final=a.lr_final, seed=a.seed,
                             loss=LOSS_ENERGY if a.loss == "energy" else LOSS_MSE)
    per_epoch = (ds.pairs - val) // a.batch * a.batch
    for e in range(a.epochs):
        print("epoch %d  train %.5f  val %.5f" % (e, tl[e], vl[e]), flush=True)
    print("training: %.1f s, %.1f samples/s" % (secs, per_epoch * a.epochs / secs), flush=True)
    ds.close()
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        net.save(a.out)
    summary = {"pairs": ds.pairs, "pair_kind": a.pairs, "grid": list(res), "generate_s": ds.seconds, "train_s": secs, "loss": a.loss,
               "epochs": a.epochs, "batch": a.batch, "train_loss": [float(v) for v in tl],
               "val_loss": [float(v) for v in vl], "eval": {}}
    return finish(a, net, summary, t0)


def finish(a, net, summary, t0):
    for spec in filter(None, a.eval_res.split(";")):
        r = tuple(int(v) for v in spec.split(","))
        ev = evaluate(net, r, a.eval_steps, precondition=a.pairs == "iterate")
        summary["eval"]["x".join(map(str, r))] = ev
        print("eval %s: plain %.1f it/step %.2f steps/s | learned %.1f it/step %.2f steps/s "
              "(fallbacks %d) | velocity rel L2 %.2e" % (
                  "x".join(map(str, r)), ev["plain"]["iters_per_step"], ev["plain"]["steps_per_s"],
                  ev["learned"]["iters_per_step"], ev["learned"]["steps_per_s"], ev["learned"]["fallbacks"],
                  ev["velocity_rel_l2"]), flush=True)
    summary["wall_s"] = time.time() - t0
    if a.log:
        with open(a.log, "w") as f:
            json.dump(summary, f, indent=1)
    net.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
