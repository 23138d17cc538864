"""Generate the long-run fixtures of the benchmark plume from the FP64 oracle.

The benchmark workload is the 128x192x128 plume (closed box, box source with
+-0.05 seeded noise, buoyancy 1 on temperature, vorticity 2) solved to a
relative L2 residual, for 200 steps.  The reference's own solvePoisson
(FLUID_3D_MIC.cpp:918-1015) can only stop on its absolute signed-max test, so
these runs use the oracle restatement (oracle/plume_oracle.cpp), whose
reference-criterion runs match the compiled reference bit for bit
(tests/test_oracle.py), with the relative-L2 stop test swapped in.

Each run stores, for every step, the PCG iteration count and the L2 norm and
sum of velocity, density, heat and pressure, and at the snapshot steps every
STRIDE-th value of those four fields (the same cells for every run):

  oracle_plume_128x192x128_tol1e-06.npz    rel-L2 1e-6 (the benchmark's test)
  oracle_plume_128x192x128_tol1e-10.npz    rel-L2 1e-10 (the converged field)

and, for the large plume of the same family (256x384x256, the box scaled the
same way), the first 12 steps at rel-L2 1e-6 with samples after steps 6 and
12, every 1021st value:

  oracle_plume_256x384x256_tol1e-06.npz

Usage: python tests/golden/make_golden_plume.py <tol> [steps] [--res X,Y,Z]
                                               [--snapshots a,b,..] [--stride n]
A 128x192x128 run takes 20-60 minutes on one core, the 256x384x256 one about
an hour; runs can go side by side.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cfs_plume_gb300 import _abi  # noqa: E402
from oracle import oracle  # noqa: E402

RES = (128, 192, 128)
STRIDE = 127
SNAPSHOTS = (20, 100, 200)
FIELDS = ("velocity", "density", "heat", "pressure")


def fixture_path(tol, res=RES):
    return os.path.join(HERE, "oracle_plume_%dx%dx%d_tol%.0e.npz" % (tuple(res) + (tol,)))


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("tol", type=float)
    ap.add_argument("steps", type=int, nargs="?", default=200)
    ap.add_argument("--res", default=",".join(str(v) for v in RES))
    ap.add_argument("--snapshots", default=",".join(str(v) for v in SNAPSHOTS))
    ap.add_argument("--stride", type=int, default=STRIDE)
    a = ap.parse_args()
    tol, steps, stride = a.tol, a.steps, a.stride
    res = tuple(int(v) for v in a.res.split(","))
    snapshots = tuple(int(v) for v in a.snapshots.split(","))
    p = _abi.plume_config(res, precision=_abi.PREC_FP64, criterion=_abi.CRIT_REL2, tol=tol)
    o = oracle.Oracle(p)
    rec = {"res": np.array(res), "tol": tol, "steps": steps, "stride": stride,
           "snapshots": np.array([s for s in snapshots if s <= steps])}
    iters, rel = [], []
    norms = {f: [] for f in FIELDS}
    sums = {f: [] for f in FIELDS}
    t0 = time.time()
    for s in range(steps):
        o.add_source(s)
        st = o.step()
        iters.append(st.iterations)
        rel.append(st.rel_residual)
        for f in FIELDS:
            a = o.field(f)
            norms[f].append(np.sqrt((a * a).sum()))
            sums[f].append(a.sum())
            if s + 1 in snapshots:
                rec["sample_%s_%d" % (f, s + 1)] = a[::stride].copy()
        print("step %d iters %d rel %.3e  %.0f s" % (s + 1, st.iterations, st.rel_residual,
                                                     time.time() - t0), flush=True)
    rec["iters"] = np.array(iters)
    rec["rel_residual"] = np.array(rel)
    for f in FIELDS:
        rec["l2_" + f] = np.array(norms[f])
        rec["sum_" + f] = np.array(sums[f])
    np.savez_compressed(fixture_path(tol, res), **rec)
    print("wrote", fixture_path(tol, res))


if __name__ == "__main__":
    main()
