"""TEST INFRASTRUCTURE ONLY: CPU restatement of the flexible-CG solve with the
network as the preconditioner stage (PLUME_PRECOND_NET, include/plume.h).

Only tests/ and the fixture generators import it; no product path does.

The reference solves with MIC(0)-PCG (FLUID_3D_MIC::solvePoisson,
FLUID_3D_MIC.cpp:918-1015); it has no flexible variant and no network, so this
module restates the algorithm the CUDA engine implements, in float64:

  r = b - A x;  z = M(r);  d = z;  delta = z.r
  loop:  q = A d;  alpha = delta / d.q;  x += alpha d;  r -= alpha q
         stop when ||r||_2 <= tol ||b||_2
         z = M(r);  beta = -(z.q) / (d.q);  delta = z.r + beta (d.r);  d = z + beta d

(Notay's FCG(1): the new direction is A-orthogonal to the last one and alpha
is the exact line search along it).  The iteration count is the number of
updates of x, as the engine reports it.  The network preconditioner is
M(r) = s c y(r / s) on interior cells, s = the RMS of r over the interior,
y the network (oracle/unet_oracle.py, BF16 rounding points) and c the scale
stored with its weights.
"""
import numpy as np

from oracle import oracle
from oracle import unet_oracle as uo


def load_net_file(path):
    """(params float64, kind, scale c) of a network file written by
    plume_net_save: "PLUMENET", int32 version and kind, int64 count, two
    float32 (scale, 0), then the float32 parameters."""
    raw = open(path, "rb").read()
    assert raw[:8] == b"PLUMENET", path
    version, kind = np.frombuffer(raw, dtype="<i4", count=2, offset=8)
    n = int(np.frombuffer(raw, dtype="<i8", count=1, offset=16)[0])
    scale = float(np.frombuffer(raw, dtype="<f4", count=2, offset=24)[0])
    params = np.frombuffer(raw, dtype="<f4", count=n, offset=32).astype(np.float64)
    assert version == 1 and params.size == uo.num_params()
    return params, int(kind), scale


def interior(res):
    X, Y, Z = res
    m = np.zeros((Z, Y, X), dtype=bool)
    m[1:-1, 1:-1, 1:-1] = True
    return m.ravel()


class NetPreconditioner:
    """z = s c y(r / s) on interior cells (0 elsewhere), as the engine's
    precondition_net applies the network (unet.cu predict)."""

    def __init__(self, path, res, bf16=True):
        params, _, self.c = load_net_file(path)
        self.net = uo.UNetOracle(params, bf16=bf16)
        self.res = tuple(res)
        self.mask = interior(res)
        self.applications = 0

    def __call__(self, r):
        m = self.mask
        s = float(np.float32(np.sqrt((r[m] ** 2).sum() / m.sum())))
        inp = np.zeros_like(r)
        if s > 0:
            inp[m] = (r[m].astype(np.float32) * np.float32(1.0 / s)).astype(np.float64)
        y, _ = self.net.forward(inp[None, :], self.res, 1)
        z = np.zeros_like(r)
        z[m] = (np.float32(s * self.c) * y[0][m].astype(np.float32)).astype(np.float64)
        self.applications += 1
        return z


class MicPreconditioner:
    """z = M^-1 r with the reference's MIC(0) (applyMICPreconditioner)."""

    def __init__(self, res, bc, tau=0.97, sigma=0.25):
        self.res, self.bc = tuple(res), tuple(bc)
        self.precon = oracle.mic_precon(self.res, self.bc, tau, sigma)

    def __call__(self, r):
        return oracle.mic_apply(self.res, self.bc, self.precon, r)[0]


def fcg(res, bc, b, precondition, tol=1e-6, max_iters=1000, x0=None):
    """Flexible CG on the interior of the full grid (reference layout); the
    stop test is ||r||_2 <= tol ||b||_2 over the interior.  Returns
    (x, iterations, relative residual history)."""
    m = interior(res)
    A = lambda v: oracle.mult_a(res, bc, v)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    bb = np.where(m, b, 0.0)
    r = np.where(m, bb - A(x), 0.0)
    bnorm = np.sqrt((bb * bb).sum())
    if bnorm == 0.0:  # nothing to solve
        return x, 0, [0.0]
    hist = [np.sqrt((r * r).sum()) / bnorm]
    if hist[-1] <= tol:
        return x, 0, hist
    z = precondition(r)
    d = z.copy()
    delta = (z * r).sum()
    for it in range(max_iters):
        q = A(d)
        dq = (d * q).sum()
        alpha = delta / dq
        x += alpha * d
        r -= alpha * q
        hist.append(np.sqrt((r * r).sum()) / bnorm)
        if hist[-1] <= tol:
            return x, it + 1, hist
        z = precondition(r)
        beta = -(z * q).sum() / dq
        delta = (z * r).sum() + beta * (d * r).sum()
        d = z + beta * d
    return x, max_iters, hist
