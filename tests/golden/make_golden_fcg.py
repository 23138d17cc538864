"""Fixture of the flexible-CG solve with the network preconditioner
(oracle/fcg_oracle.py) on a right-hand side of the 48x64x48 benchmark plume.

The right-hand side is the divergence after STEPS steps of the FP64 oracle
(closed box, box source with seeded noise, buoyancy 1, vorticity 2), which the
GPU test recomputes the same way.  Stored: the iteration counts of FCG with the
committed network and with MIC(0) as M (equal to MIC-PCG's), the relative
residual histories, and every STRIDE-th value of the FCG-network solution.

Usage: python tests/golden/make_golden_fcg.py      (about a minute)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cfs_plume_gb300 import _abi  # noqa: E402
from oracle import fcg_oracle as fo  # noqa: E402
from oracle import oracle  # noqa: E402

RES = (48, 64, 48)
STEPS = 10
STRIDE = 5
TOL = 1e-6
WEIGHTS = os.path.join(ROOT, "cfs_plume_gb300", "weights", "unet_warmstart.bin")
OUT = os.path.join(HERE, "oracle_fcg_48x64x48.npz")


def rhs():
    p = _abi.plume_config(RES, precision=_abi.PREC_FP64)
    o = oracle.Oracle(p)
    for s in range(STEPS):
        o.add_source(s)
        o.step()
    return p, o.field("divergence")


def main():
    p, b = rhs()
    bc = tuple(p.bc)
    x, it, hist = fo.fcg(RES, bc, b, fo.NetPreconditioner(WEIGHTS, RES), tol=TOL)
    xm, itm, histm = fo.fcg(RES, bc, b, fo.MicPreconditioner(RES, bc), tol=TOL)
    np.savez_compressed(OUT, res=np.array(RES), steps=STEPS, tol=TOL, stride=STRIDE,
                        iters_net=it, hist_net=np.array(hist), iters_mic=itm, hist_mic=np.array(histm),
                        x_net=x[::STRIDE].copy(), x_mic=xm[::STRIDE].copy(), b_l2=np.linalg.norm(b))
    print("FCG iterations: network", it, "MIC(0)", itm, "->", OUT)


if __name__ == "__main__":
    main()
