"""Wall time of the warm-start network's forward pass (host input in, host
output out) at one grid size: `warmup` untimed passes, then `iters` timed
ones, on a seeded standard-normal field.

    python -m cfs_plume_gb300.bench_net [--res 128,192,128] [--warmup 3] [--iters 5]

PLUME_CONV_TC=0 in the environment runs every convolution on the mma.sync
kernel instead of tcgen05 where both exist.
"""
import argparse
import json
import os
import time

import numpy as np

from .net import PlumeNet

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", default="128,192,128")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--weights", default=os.path.join(HERE, "weights", "unet_warmstart.bin"))
    a = ap.parse_args()
    res = tuple(int(v) for v in a.res.split(","))
    net = PlumeNet(seed=0, path=a.weights)
    x = np.random.default_rng(0).standard_normal((1, res[2], res[1], res[0])).astype(np.float32)
    for _ in range(a.warmup):
        net.forward(x, res)
    t0 = time.perf_counter()
    for _ in range(a.iters):
        y = net.forward(x, res)
    ms = (time.perf_counter() - t0) / max(1, a.iters) * 1000.0
    net.close()
    print(json.dumps({"res": res, "forward_ms_wall": ms, "mean_abs_output": float(np.abs(y).mean()),
                      "tcgen05": os.environ.get("PLUME_CONV_TC", "1") != "0"}))


if __name__ == "__main__":
    main()
