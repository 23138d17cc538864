"""The FP32 MIC(0) sweeps' form of applyMICPreconditioner
(FLUID_3D_MIC.cpp:864-899), restated in FP64 and checked against the oracle
on the CPU: the diagonal is used squared, the forward sweep's intermediate is
w = P q instead of q, and

    forward   w = P^2 (r + w[-x] + w[-y] + w[-z])
    backward  z = w + P^2 (z[+x] + z[+y] + z[+z])

(from q = P (r + sum P q[-]) and z = P (q + P sum z[+]), the plume's
off-diagonal entries being -1 between interior cells).  The CUDA sweeps
(wave.cuh, sweep_cell without EXACT) evaluate exactly this in FP32; here it
must equal the reference's operator to rounding.  No GPU needed."""
import numpy as np
import pytest

from oracle import oracle


def _interior(a, res):
    return a.reshape(res[::-1])[1:-1, 1:-1, 1:-1]


def _sweeps_p2(P, r):
    nz, ny, nx = r.shape
    P2 = P * P
    w = np.zeros_like(r)
    z = np.zeros_like(r)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                s = r[k, j, i]
                s += w[k, j, i - 1] if i else 0.0
                s += w[k, j - 1, i] if j else 0.0
                s += w[k - 1, j, i] if k else 0.0
                w[k, j, i] = P2[k, j, i] * s
    for k in reversed(range(nz)):
        for j in reversed(range(ny)):
            for i in reversed(range(nx)):
                s = z[k, j, i + 1] if i + 1 < nx else 0.0
                s += z[k, j + 1, i] if j + 1 < ny else 0.0
                s += z[k + 1, j, i] if k + 1 < nz else 0.0
                z[k, j, i] = w[k, j, i] + P2[k, j, i] * s
    return z, w


@pytest.mark.parametrize("res,bc", [((10, 11, 9), (1, 1, 1, 1, 1, 1)), ((9, 12, 8), (0, 0, 0, 0, 0, 0)),
                                    ((12, 8, 10), (1, 0, 1, 0, 1, 0))])
def test_p2_sweeps_equal_the_reference_operator(res, bc):
    rng = np.random.default_rng(17)
    n = res[0] * res[1] * res[2]
    r = np.zeros(n)
    _interior(r, res)[...] = rng.standard_normal(tuple(v - 2 for v in res[::-1]))
    prec = oracle.mic_precon(res, bc)
    zo, qo = oracle.mic_apply(res, bc, prec, r)
    z, w = _sweeps_p2(_interior(prec, res), _interior(r, res))
    zi, qi, Pi = _interior(zo, res), _interior(qo, res), _interior(prec, res)
    assert np.abs(z - zi).max() <= 1e-12 * np.abs(zi).max()
    assert np.abs(w - Pi * qi).max() <= 1e-12 * np.abs(Pi * qi).max()
