"""The projected-operator build of a reduced model (buildOutOfCoreMatrices,
plume_reduced_build_products) on seeded synthetic bases: `warmup` untimed
builds, then `iters` timed ones; prints the device and wall times and the
FP64 rate of the last build.

    python -m cfs_plume_gb300.bench_products [--res 64,96,64] [--rank 32]
                                             [--warmup 1] [--iters 1]

The bases are standard-normal columns scaled by 1/sqrt(rows): U.pressure has
N_int rows, U.preproject, U.prediffuse and U.final 3 N_int, each `rank`
columns, written in the reference's matrix file layout to a temporary
reduced path; the walls are the reference defaults.
"""
import argparse
import json
import math
import os
import shutil
import struct
import tempfile

import numpy as np

from . import _abi
from .plume import Plume, build_products


def write_matrix(path, M):
    """EIGEN::write layout: int32 rows, cols, then the row-major doubles."""
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", M.shape[0], M.shape[1]))
        M.astype("<f8").tofile(f)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", default="64,96,64")
    ap.add_argument("--rank", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--iters", type=int, default=1)
    a = ap.parse_args()
    res = tuple(int(v) for v in a.res.split(","))
    nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
    rng = np.random.default_rng(11)
    d = tempfile.mkdtemp(prefix="plume_products_") + "/"
    try:
        write_matrix(d + "U.pressure.matrix", rng.standard_normal((nint, a.rank)) / math.sqrt(nint))
        for fn in ("U.preproject.matrix", "U.prediffuse.matrix", "U.final.matrix"):
            write_matrix(d + fn, rng.standard_normal((3 * nint, a.rank)) / math.sqrt(3 * nint))
        g = Plume(_abi.default_params(res=res))
        for _ in range(a.warmup):
            build_products(g, d)
        dev = wall = 0.0
        info = None
        for _ in range(a.iters):
            info = build_products(g, d)
            dev += info["ms_device"]
            wall += info["ms_total"]
        g.close()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    n = max(1, a.iters)
    print(json.dumps({"res": res, "rank": a.rank, "ms_device": dev / n, "ms_total": wall / n,
                      "gflop": info["gflop"], "tflops": info["gflop"] / (dev / n) if dev > 0 else None}))


if __name__ == "__main__":
    main()
