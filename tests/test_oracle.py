"""CPU tests: the oracle restatement is pinned to the reference's own outputs.

The fixtures under tests/golden/ were produced by the reference's unmodified
FLUID_3D_MIC.cpp (tests/golden/make_golden.py).  The oracle must reproduce
every state field bit for bit and the PCG iteration count of every step.
"""
import glob
import os

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import oracle
from tests.state_format import read_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _params_from(z, **extra):
    kw = dict(res=tuple(int(v) for v in z["res"]), bc=tuple(int(v) for v in z["bc"]),
              buoyancy=float(z["buoyancy"]), vorticity_eps=float(z["vorticity_eps"]),
              source=int(z["source"]), box_lo=tuple(int(v) for v in z["box_lo"]),
              box_hi=tuple(int(v) for v in z["box_hi"]), source_noise=float(z["source_noise"]),
              seed=int(z["seed"]))
    kw.update(extra)
    return _abi.default_params(**kw)


def run_oracle(p, steps):
    o = oracle.Oracle(p)
    iters = []
    for s in range(steps):
        o.add_source(s)
        iters.append(o.step().iterations)
    return o, iters


CASES = sorted(os.path.basename(f)[4:-4] for f in glob.glob(os.path.join(GOLDEN, "ref_*.npz"))
               if not any(k in os.path.basename(f) for k in ("sampled", "moving", "svd", "reduced", "products")))


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_bit_for_bit(case):
    z = np.load(os.path.join(GOLDEN, "ref_%s.npz" % case))
    p = _params_from(z)
    o, iters = run_oracle(p, int(z["steps"]))
    assert iters == list(z["iters"]), "PCG iteration counts differ from the reference"
    for name in _abi.FIELDS:
        a = o.field(name)
        assert np.array_equal(a, z[name]), "field %s differs (max %.3e)" % (
            name, np.abs(a - z[name]).max())
    assert np.array_equal(o.obstacles(), z["obstacles"])


def test_oracle_benchmark_plume_48x64x48():
    """The 48x64x48 plume (box source, closed box, FP64, 1e-10): iteration
    counts, per-field sums/norms and a strided sample match the reference."""
    z = np.load(os.path.join(GOLDEN, "ref_cfg1_sampled.npz"))
    p = _params_from(z, precision=_abi.PREC_FP64, criterion=_abi.CRIT_REFERENCE, tol=1e-10)
    o, iters = run_oracle(p, int(z["steps"]))
    assert iters == list(z["iters"])
    for name in _abi.FIELDS:
        a = o.field(name)
        assert np.array_equal(a[::97], z["sample_" + name]), name
        assert a.sum() == z["sum_" + name], name
        assert np.sqrt((a * a).sum()) == z["l2_" + name], name


def test_reference_state_file_layout():
    """The reference's own state file parses with the test reader and holds the
    fields the reference's readGz returned."""
    d = os.path.join(GOLDEN, "ref_state_8x10x6")
    s = read_state(os.path.join(d, "fluid.0001.fluid3d.gz"))
    f = np.load(os.path.join(d, "fields.npz"))
    ints = s["header_ints"]
    assert ints[:3] == (8, 10, 6) and ints[4:7] == (1, 8, 80) and ints[7] == 480 and ints[9] == 2
    for name in _abi.FIELDS:
        assert np.array_equal(s[name], f[name]), name
    assert s["iop_count"] == 0
    assert s["midMaccormack_meta"][0] == (0, 0, 0)
    assert s["trailing_bytes"] == 0


def test_reference_streams_layout():
    """appendStreams rows: peeled interior, x fastest, components interleaved;
    pressure and divergence share one stream; dims = (rows, cols)."""
    d = os.path.join(GOLDEN, "ref_state_8x10x6")
    f = np.load(os.path.join(d, "fields.npz"))
    res = (8, 10, 6)
    nint = 6 * 8 * 4

    def dims(name):
        return tuple(np.fromfile(os.path.join(d, name + ".matrix.dims"), dtype="<i4"))

    assert dims("velocity.final") == (2, 3 * nint)
    assert dims("velocity.iop") == (0, 3 * nint)
    assert dims("pressure") == (4, nint)
    rows = np.fromfile(os.path.join(d, "velocity.final.matrix.transpose")).reshape(2, -1)
    v = f["velocity"].reshape(res[2], res[1], res[0], 3)[1:-1, 1:-1, 1:-1].ravel()
    assert np.array_equal(rows[1], v)
    pr = np.fromfile(os.path.join(d, "pressure.matrix.transpose")).reshape(4, -1)
    assert np.array_equal(pr[2], f["pressure"].reshape(res[::-1])[1:-1, 1:-1, 1:-1].ravel())
    assert np.array_equal(pr[3], f["divergence"].reshape(res[::-1])[1:-1, 1:-1, 1:-1].ravel())


def test_rel2_criterion_reaches_tolerance():
    """The rel-L2 mode (restated for the 1e-6 configurations) stops with the
    true residual at or below the tolerance."""
    res = (20, 24, 18)
    p = _abi.plume_config(res, precision=_abi.PREC_FP64)
    o, iters = run_oracle(p, 4)
    assert all(i > 0 for i in iters)
    b = o.field("divergence")
    x = o.field("pressure")
    r = b - oracle.mult_a(res, tuple(p.bc), x)
    inner = np.zeros(res[::-1], dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    inner = inner.ravel()
    rel = np.linalg.norm(r[inner]) / np.linalg.norm(b[inner])
    assert rel <= 1.0001e-6


def test_source_noise_is_seeded_and_bounded():
    vals = np.array([oracle.source_value(3, 5, c, 0.05) for c in range(2000)])
    assert np.all(np.abs(vals - 1.0) <= 0.05)
    assert vals.std() > 0.02
    again = np.array([oracle.source_value(3, 5, c, 0.05) for c in range(2000)])
    assert np.array_equal(vals, again)
    other = np.array([oracle.source_value(4, 5, c, 0.05) for c in range(2000)])
    assert not np.array_equal(vals, other)
