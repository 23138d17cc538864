"""Batched-plume throughput: 64 independent randomised plumes on one GPU.

    python -m cfs_plume_gb300.bench_batch [--n 64] [--steps 100] [--warmup 3]

Instances come from plume_batch_params (grids drawn from 32^3 .. 96x128x96,
randomised source position, buoyancy and vorticity, FP32 fields, rel-L2 1e-6)
and advance concurrently (one handle and CUDA stream each, host thread pool).
Prints one JSON line: aggregate interior cell-steps/s over the timed steps,
and the same batch stepped one instance after another for comparison.
"""
import argparse
import json
import sys

import numpy as np

from .batch import PlumeBatch, batch_params


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0, help="host threads (0: one per instance)")
    ap.add_argument("--serial-steps", type=int, default=10, help="steps of the one-at-a-time comparison")
    a = ap.parse_args(argv)
    params = [batch_params(a.seed, i) for i in range(a.n)]
    cells = np.array([(p.res[0] - 2) * (p.res[1] - 2) * (p.res[2] - 2) for p in params], dtype=np.float64)
    b = PlumeBatch(params)
    b.run(0, a.warmup, threads=a.threads, stats=False)
    secs, stats = b.run(a.warmup, a.steps, threads=a.threads, stats=True)
    iters = np.array([[s.iterations for s in st] for st in stats], dtype=np.float64)
    conv = all(s.converged for st in stats for s in st)
    value = cells.sum() * a.steps / secs
    serial = None
    if a.serial_steps > 0:
        s_secs, _ = b.run(a.warmup + a.steps, a.serial_steps, threads=1, stats=False)
        serial = cells.sum() * a.serial_steps / s_secs
    b.close()
    grids = {}
    for p in params:
        k = "x".join(str(v) for v in p.res)
        grids[k] = grids.get(k, 0) + 1
    line = {"metric": "aggregate interior cell-steps/s, batched plumes", "value": value,
            "unit": "cell-steps/s", "instances": a.n, "steps": a.steps, "warmup": a.warmup,
            "seconds": secs, "instance_steps_per_s": a.n * a.steps / secs,
            "pcg_iters_per_step_mean": float(iters.mean()), "all_converged": conv,
            "grids": grids, "interior_cells_total": float(cells.sum()),
            "one_at_a_time": {"value": serial, "steps": a.serial_steps},
            "config": {"workload": "%d randomised closed-box plumes (batched-plume configuration), "
                                   "FP32 fields, MIC(0)-PCG rel-L2 1e-6" % a.n,
                       "threads": a.threads or a.n}}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
