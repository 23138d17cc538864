"""The moving box obstacle (include/plume_box.h): FLUID_3D_MIC::
stepWithMovingObstacle, setPeeledSparseMovingIOP, setInitialVelocity(BOX*)
and the BOX motion.

CPU: the oracle restatement against the reference's own outputs (fixtures
made by tests/golden/make_golden.py from the reference's FLUID_3D_MIC.cpp),
the reference's state-file and stream layout of a moving run, and the
product's host-side box motion against the oracle's, bit for bit.

GPU (through the C ABI), tolerances as in test_gpu_parity.py:
 * FP64 with the solver disabled (max_iters = 0): every field, postIOP and
   the obstacle matrix bit-identical to the oracle, step after step;
 * FP64 full steps: fields to a relative L2 of 1e-9 of the reference's
   fixtures, PCG iterations within one; the obstacle matrix bit-identical
   (it depends on the box alone);
 * FP32: relative L2 against the FP64 oracle, bound stated in the test.
"""
import ctypes as C
import math
import os

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import oracle
from tests.state_format import read_sparse_matrices, read_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MOVING = ["box_16x20x12", "box_open_14x12x16"]


def _fixture(case):
    return np.load(os.path.join(GOLDEN, "ref_moving_%s.npz" % case))


def _params_from(z, **extra):
    kw = dict(res=tuple(int(v) for v in z["res"]), bc=tuple(int(v) for v in z["bc"]),
              buoyancy=float(z["buoyancy"]), vorticity_eps=float(z["vorticity_eps"]),
              source=int(z["source"]), box_lo=tuple(int(v) for v in z["box_lo"]),
              box_hi=tuple(int(v) for v in z["box_hi"]), source_noise=float(z["source_noise"]),
              seed=int(z["seed"]))
    kw.update(extra)
    return _abi.default_params(**kw)


def _oracle_box(z):
    b = oracle.box_init(tuple(z["box_center"]), tuple(z["box_lengths"]), float(z["period"]),
                        float(z["translation_period"]))
    b.dt = 0.1  # BOX::set_dt in lock-step with the fluid
    return b


def run_oracle_moving(z, steps=None, **extra):
    p = _params_from(z, **extra)
    o = oracle.Oracle(p)
    b = _oracle_box(z)
    if int(z["initvel"]):
        o.set_initial_velocity_box(b)
    iters = []
    for s in range(int(z["steps"]) if steps is None else steps):
        o.add_source(s)
        iters.append(o.step_moving_box(b).iterations)
        oracle.box_spin(b)
        oracle.box_translate(b)
    return o, iters


def _iop_from_mask(res, inside, values):
    """Map-ordered (row, col) pairs and values of the obstacle matrix from the
    full-grid inside mask and last-column values (plume_download_iop)."""
    X, Y, Z = res
    rows = 3 * (X - 2) * (Y - 2) * (Z - 2)
    ij, val = [], []
    m = inside.reshape(Z, Y, X)[1:-1, 1:-1, 1:-1].ravel()
    v = values.reshape(Z, Y, X, 3)[1:-1, 1:-1, 1:-1].reshape(-1, 3)
    for c in range(m.size):
        for i in range(3):
            r = 3 * c + i
            if m[c]:
                ij += [(r, r), (r, rows)]
                val += [0.0, v[c, i]]
            else:
                ij.append((r, r))
                val.append(1.0)
    return (rows, rows + 1), np.array(ij, dtype=np.int32), np.array(val)


# ------------------------------------------------------------------ CPU tests
@pytest.mark.parametrize("case", MOVING)
def test_oracle_moving_step_matches_reference_bit_for_bit(case):
    z = _fixture(case)
    o, iters = run_oracle_moving(z)
    assert iters == list(z["iters"])
    for name in _abi.FIELDS + ["postIOP"]:
        a = o.field(name)
        assert np.array_equal(a, z[name]), "%s differs (max %.3e)" % (name, np.abs(a - z[name]).max())
    dims, ij, val = o.iop_entries()
    assert dims == tuple(z["iop_dims"])
    assert np.array_equal(ij, z["iop_ij"])
    assert np.array_equal(val.view(np.uint64), z["iop_val"].view(np.uint64))


def test_moving_fixture_covers_wraps_and_partial_box():
    """The open-face case spins and sways fast enough that theta and phi pass
    2 pi within its 8 steps, and its box reaches out of the domain."""
    z = _fixture("box_open_14x12x16")
    b = _oracle_box(z)
    wraps_t = wraps_p = 0
    for _ in range(int(z["steps"])):
        t, ph = b.theta, b.phi
        oracle.box_spin(b)
        oracle.box_translate(b)
        wraps_t += b.theta < t
        wraps_p += b.phi < ph
    assert wraps_t >= 1 and wraps_p >= 1
    c, l = z["box_center"], z["box_lengths"]
    assert c[0] + 0.5 * l[0] > 1.0
    inside = (z["iop_val"][z["iop_ij"][:, 0] == z["iop_ij"][:, 1]] == 0.0).sum()
    assert inside > 0


def test_reference_moving_state_file_layout():
    """A moving run's state file: postIOP with the grid's dims, then the
    obstacle matrix (rows 3 n_int, cols 3 n_int + 1) in (row, col) order with
    one diagonal entry per row, 0 and a last-column entry inside the box."""
    d = os.path.join(GOLDEN, "ref_moving_state_10x12x8")
    s = read_state(os.path.join(d, "fluid.0001.fluid3d.gz"))
    res = (10, 12, 8)
    nint = 8 * 10 * 6
    assert s["postIOP_meta"][0] == res
    assert s["iop_dims"] == (3 * nint, 3 * nint + 1)
    ij, val = s["iop_ij"], s["iop_val"]
    key = ij[:, 0].astype(np.int64) * (3 * nint + 1) + ij[:, 1]
    assert np.all(np.diff(key) > 0)
    diag = ij[:, 0] == ij[:, 1]
    assert diag.sum() == 3 * nint
    last = ij[:, 1] == 3 * nint
    assert np.all(diag | last)
    inside_rows = set(ij[last, 0])
    assert np.all(val[diag & np.isin(ij[:, 0], list(inside_rows))] == 0.0)
    assert np.all(val[diag & ~np.isin(ij[:, 0], list(inside_rows))] == 1.0)
    assert s["trailing_bytes"] == 0
    mats = read_sparse_matrices(os.path.join(d, "neumann.iop.matrices"))
    assert len(mats) == 2  # one per appendStreams call
    assert np.array_equal(mats[1][1], ij) and np.array_equal(mats[1][2], val)
    rows, cols = np.fromfile(os.path.join(d, "velocity.iop.matrix.dims"), dtype="<i4")
    assert (rows, cols) == (2, 3 * nint)


def deinterleave_reference_iop_rows(raw, row_len):
    """The reference never closes the FILE of velocity.iop.matrix.transpose
    in appendStreams (opened at FLUID_3D_MIC.cpp:1385; the fclose list at
    1458-1463 leaves it out), so each call's row reaches the file in two
    parts: what stdio wrote through at the fwrite (the largest multiple of
    its 4096-byte buffer, 8192 of the 11520 bytes here) and the buffered rest
    at process exit, newest stream first.  The committed fixture (two rows)
    therefore holds row0[:1024] row1 row0[1024:]; this undoes that."""
    head = (row_len * 8 // 4096) * 4096 // 8
    assert raw.size == 2 * row_len
    return np.stack([np.concatenate([raw[:head], raw[head + row_len:]]), raw[head:head + row_len]])


def test_reference_iop_stream_rows_are_the_postiop_rows_out_of_order():
    """The reference's own IOP stream, de-interleaved, is the peeled postIOP
    of each step bit for bit (the oracle's); a writer that closes its file
    (this library's) appends the same rows in step order."""
    d = os.path.join(GOLDEN, "ref_moving_state_10x12x8")
    zb = np.load(os.path.join(d, "box.npz"))
    raw = np.fromfile(os.path.join(d, "velocity.iop.matrix.transpose"))
    rows = deinterleave_reference_iop_rows(raw, 3 * 8 * 10 * 6)
    for s in range(2):
        o, _ = run_oracle_moving(zb, steps=s + 1)
        peeled = o.field("postIOP").reshape(8, 12, 10, 3)[1:-1, 1:-1, 1:-1].ravel()
        assert np.array_equal(rows[s], peeled), s
    assert not np.array_equal(raw[:rows.shape[1]], rows[0])  # the raw file is out of order


def test_oracle_reproduces_reference_moving_state_file():
    d = os.path.join(GOLDEN, "ref_moving_state_10x12x8")
    zb = np.load(os.path.join(d, "box.npz"))
    s = read_state(os.path.join(d, "fluid.0001.fluid3d.gz"))
    o, _ = run_oracle_moving(zb, steps=2)
    for name in _abi.FIELDS + ["postIOP"]:
        assert np.array_equal(o.field(name), s[name]), name
    dims, ij, val = o.iop_entries()
    assert dims == s["iop_dims"] and np.array_equal(ij, s["iop_ij"])
    assert np.array_equal(val, s["iop_val"])


def _product_box(lib, center, lengths, period, tperiod):
    b = _abi.PlumeBox()
    assert lib.plume_box_init(C.byref(b), (C.c_double * 3)(*center), (C.c_double * 3)(*lengths),
                              period, tperiod) == 0
    return b


def _box_bytes(b):
    return bytes(memoryview(b))


@pytest.mark.parametrize("period,tperiod", [(4.0, 8.0), (0.45, 0.35), (1.0 / 3.0, 0.7)])
def test_product_box_motion_matches_oracle_bit_for_bit(plume_lib, period, tperiod):
    """plume_box_init / spin / translate / inside / velocity against the
    oracle's restatement of BOX: the whole struct bit for bit over 100 steps,
    inside and velocity at seeded points around the box."""
    from cfs_plume_gb300 import plume as P
    P.load_library()
    lib = plume_lib
    c, l = (0.45, 0.4, 0.55), (0.3, 0.2, 0.35)
    a = _product_box(lib, c, l, period, tperiod)
    b = oracle.box_init(c, l, period, tperiod)
    assert _box_bytes(a) == _box_bytes(b)
    a.dt = b.dt = 0.1
    rng = np.random.default_rng(5)
    for _ in range(100):
        assert lib.plume_box_spin(C.byref(a)) == 0
        assert lib.plume_box_translate(C.byref(a)) == 0
        oracle.box_spin(b)
        oracle.box_translate(b)
        assert _box_bytes(a) == _box_bytes(b)
        for p in rng.uniform(0.0, 1.0, size=(8, 3)):
            pt = (C.c_double * 3)(*p)
            ins = C.c_int32()
            assert lib.plume_box_inside(C.byref(a), pt, C.byref(ins)) == 0
            assert bool(ins.value) == oracle.box_inside(b, p)
            v = (C.c_double * 3)()
            assert lib.plume_box_velocity(C.byref(a), pt, v) == 0
            assert np.array_equal(np.array(v[:]), np.array(oracle.box_velocity(b, p)))


def test_box_facade_names(plume_lib):
    from cfs_plume_gb300.plume import BOX
    box = BOX((0.5, 0.5, 0.5), (0.2, 0.2, 0.2), 4.0, 8.0)
    assert box.inside((0.5, 0.5, 0.5)) and not box.inside((0.9, 0.5, 0.5))
    box.set_dt(0.1)
    box.spin()
    box.translate_center()
    assert box.theta == 2 * math.pi * 0.1 / 4.0
    assert box.center[0] == 0.5 + 0.25 * math.sin(2 * math.pi * 0.1 / 8.0)


def test_box_invalid_arguments(plume_lib):
    assert plume_lib.plume_box_init(None, None, None, 1.0, 1.0) == _abi.ERR_INVALID
    assert plume_lib.plume_box_spin(None) == _abi.ERR_INVALID
    assert plume_lib.plume_step_moving_box(None, None, None) == _abi.ERR_INVALID
    assert plume_lib.plume_download_iop(None, None, None, 0) == _abi.ERR_INVALID


# ------------------------------------------------------------------ GPU tests
def rel_l2(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def _gpu_box(z):
    from cfs_plume_gb300.plume import BOX
    b = BOX(tuple(z["box_center"]), tuple(z["box_lengths"]), float(z["period"]),
            float(z["translation_period"]))
    b.set_dt(0.1)
    return b


def run_gpu_moving(z, steps=None, **extra):
    from cfs_plume_gb300.plume import Plume
    g = Plume(_params_from(z, **extra))
    b = _gpu_box(z)
    if int(z["initvel"]):
        g.set_initial_velocity_box(b)
    iters = []
    for s in range(int(z["steps"]) if steps is None else steps):
        g.add_source(s)
        iters.append(g.step_moving_box(b).iterations)
        b.spin()
        b.translate_center()
    return g, iters


@pytest.mark.gpu
@pytest.mark.parametrize("case", MOVING)
def test_moving_stages_bit_exact_fp64(case):
    """Solver disabled: walls, vorticity, advection, damping, the obstacle
    stomp (postIOP), divergence and gradient bit-identical to the oracle; the
    obstacle matrix bit-identical too."""
    z = _fixture(case)
    g, gi = run_gpu_moving(z, max_iters=0)
    o, oi = run_oracle_moving(z, max_iters=0)
    assert gi == oi == [0] * int(z["steps"])
    for name in _abi.FIELDS + ["postIOP"]:
        a, b = g.field(name), o.field(name)
        assert np.array_equal(a, b), "%s differs: max |d| = %.3e" % (name, np.abs(a - b).max())
    inside, vals = g.iop()
    dims, ij, val = _iop_from_mask(tuple(z["res"]), inside, vals)
    odims, oij, oval = o.iop_entries()
    assert dims == odims and np.array_equal(ij, oij)
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("case", MOVING)
def test_moving_full_step_fp64_matches_reference_fixtures(case):
    z = _fixture(case)
    g, iters = run_gpu_moving(z)
    assert max(abs(a - b) for a, b in zip(iters, z["iters"])) <= 1, (iters, list(z["iters"]))
    for name in _abi.FIELDS + ["postIOP"]:
        err = rel_l2(g.field(name), z[name])
        assert err < 1e-9, "%s rel L2 %.3e" % (name, err)
    inside, vals = g.iop()
    dims, ij, val = _iop_from_mask(tuple(z["res"]), inside, vals)
    assert dims == tuple(z["iop_dims"]) and np.array_equal(ij, z["iop_ij"])
    assert np.array_equal(val.view(np.uint64), z["iop_val"].view(np.uint64))


@pytest.mark.gpu
def test_set_initial_velocity_box_bit_exact():
    from cfs_plume_gb300.plume import Plume
    z = _fixture("box_16x20x12")
    p = _params_from(z)
    g = Plume(p)
    o = oracle.Oracle(p)
    g.set_initial_velocity_box(_gpu_box(z))
    o.set_initial_velocity_box(_oracle_box(z))
    assert np.array_equal(g.field("velocity"), o.field("velocity"))
    assert np.abs(o.field("velocity")).max() > 0


@pytest.mark.gpu
def test_moving_fp32_against_fp64_oracle():
    """FP32 fields, FP64 CG scalars, rel-residual 1e-6, against the FP64
    oracle at the same residual: 40x48x36 closed box, box source, 12 moving
    steps.  Bound: 1e-3 relative L2 on velocity, postIOP and density (as for
    the plain step); the obstacle mask is the same (its geometry is FP64)."""
    from cfs_plume_gb300.plume import BOX, Plume
    res = (40, 48, 36)
    pg = _abi.plume_config(res, precision=_abi.PREC_FP32)
    po = _abi.plume_config(res, precision=_abi.PREC_FP64)
    g = Plume(pg)
    o = oracle.Oracle(po)
    bg = BOX((0.5, 0.45, 0.5), (0.3, 0.15, 0.25), 3.0, 5.0)
    bg.set_dt(0.1)
    bo = oracle.box_init((0.5, 0.45, 0.5), (0.3, 0.15, 0.25), 3.0, 5.0)
    bo.dt = 0.1
    for s in range(12):
        g.add_source(s)
        o.add_source(s)
        assert g.step_moving_box(bg).converged == 1
        o.step_moving_box(bo)
        bg.spin()
        bg.translate_center()
        oracle.box_spin(bo)
        oracle.box_translate(bo)
    for name in ("velocity", "postIOP", "density"):
        e = rel_l2(g.field(name), o.field(name))
        print("fp32 moving vs fp64 oracle: %s %.3e" % (name, e))
        assert e < 1e-3, name
    inside, vals = g.iop()
    dims, gij, gval = _iop_from_mask(res, inside, vals)
    odims, oij, oval = o.iop_entries()
    assert dims == odims and np.array_equal(gij, oij) and np.array_equal(gval, oval)


def _mask_numpy(res, b):
    """BOX::inside at every cell centre, elementwise in the reference's
    operation order (numpy rounds each operation separately)."""
    X, Y, Z = res
    z, y, x = np.meshgrid(np.arange(Z, dtype=np.float64), np.arange(Y, dtype=np.float64),
                          np.arange(X, dtype=np.float64), indexing="ij")
    dx, dy, dz = 1.0 / X, 1.0 / Y, 1.0 / Z
    p = [(0.0 + x * dx) + dx * 0.5, (0.0 + y * dy) + dy * 0.5, (0.0 + z * dz) + dz * 0.5]
    u = [p[k] - b.center[k] for k in range(3)]
    R = b.rotation
    ok = np.ones_like(x, dtype=bool)
    for r in range(3):
        q = (R[3 * r] * u[0] + R[3 * r + 1] * u[1]) + R[3 * r + 2] * u[2]
        ok &= np.abs(q) <= b.lengths[r] * 0.5
    ok[0, :, :] = ok[-1, :, :] = False
    ok[:, 0, :] = ok[:, -1, :] = False
    ok[:, :, 0] = ok[:, :, -1] = False
    return ok.ravel().astype(np.uint8)


@pytest.mark.gpu
def test_moving_step_full_size_properties():
    """128x192x128 FP32, the benchmark plume with a spinning box: the obstacle
    mask equals BOX::inside evaluated on every cell (so the kernel's bounding
    cell range loses no cell), postIOP equals the box velocity inside and
    the damped velocity (preprojection) outside, and every solve converges."""
    from cfs_plume_gb300.plume import BOX, Plume
    res = (128, 192, 128)
    g = Plume(_abi.plume_config(res, precision=_abi.PREC_FP32))
    box = BOX((0.5, 0.3, 0.5), (0.35, 0.1, 0.2), 2.0, 4.0)
    box.set_dt(0.1)
    for s in range(3):
        box.spin()
        box.translate_center()
        g.add_source(s)
        assert g.step_moving_box(box).converged == 1
    inside, vals = g.iop()
    assert np.array_equal(inside, _mask_numpy(res, box.state))
    assert inside.sum() > 1000
    post = g.field("postIOP").reshape(-1, 3)
    pre = g.field("preprojection").reshape(-1, 3)
    m = inside.astype(bool)
    assert np.array_equal(post[m], vals[m].astype(np.float32).astype(np.float64))
    interior = np.zeros(res[::-1], dtype=bool)
    interior[1:-1, 1:-1, 1:-1] = True
    out = interior.ravel() & ~m
    assert np.array_equal(post[out], pre[out])


@pytest.mark.gpu
def test_moving_state_file_and_streams_match_reference(tmp_path):
    """State file and streams of a moving run against the reference's own
    (10x12x8, 2 steps): same header and field metadata, fields to 1e-9, the
    obstacle matrix in the state file and in neumann.iop.matrices identical,
    the postIOP stream rows to 1e-9; the asynchronous writer gives the same."""
    import gzip
    from cfs_plume_gb300.plume import Plume
    fx = os.path.join(GOLDEN, "ref_moving_state_10x12x8")
    zb = np.load(os.path.join(fx, "box.npz"))
    d = str(tmp_path / "sync") + "/"
    da = str(tmp_path / "async") + "/"
    os.makedirs(d)
    os.makedirs(da)
    hs = [Plume(_params_from(zb)), Plume(_params_from(zb))]
    boxes = [_gpu_box(zb), _gpu_box(zb)]
    for h, b in zip(hs, boxes):
        h.set_initial_velocity_box(b)
    for s in range(2):
        for h, b in zip(hs, boxes):
            h.add_source(s)
            h.step_moving_box(b)
            b.spin()
            b.translate_center()
        hs[0].append_streams(d)
        hs[1].snapshot_async(da, s)
    hs[0].write_state(d + "fluid.0001.fluid3d")
    hs[1].wait_snapshots()
    s = read_state(d + "fluid.0001.fluid3d.gz")
    ref = read_state(os.path.join(fx, "fluid.0001.fluid3d.gz"))
    assert s["header_ints"] == ref["header_ints"] and s["header_doubles"] == ref["header_doubles"]
    for name in _abi.FIELDS + ["postIOP"]:
        assert s[name + "_meta"] == ref[name + "_meta"], name
        assert rel_l2(s[name], ref[name]) < 1e-9, name
    assert s["iop_dims"] == ref["iop_dims"] and np.array_equal(s["iop_ij"], ref["iop_ij"])
    assert np.array_equal(s["iop_val"], ref["iop_val"])
    assert s["trailing_bytes"] == 0
    ma = read_sparse_matrices(d + "neumann.iop.matrices")
    mb = read_sparse_matrices(os.path.join(fx, "neumann.iop.matrices"))
    assert len(ma) == len(mb) == 2
    for a, b in zip(ma, mb):
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    for name in ("velocity.final", "velocity.preproject", "velocity.prediffuse",
                 "velocity.preadvect", "velocity.iop", "pressure"):
        a = np.fromfile(d + name + ".matrix.dims", dtype="<i4")
        b = np.fromfile(os.path.join(fx, name + ".matrix.dims"), dtype="<i4")
        assert np.array_equal(a, b), name
        ra = np.fromfile(d + name + ".matrix.transpose")
        rb = np.fromfile(os.path.join(fx, name + ".matrix.transpose"))
        if name == "velocity.iop":  # the reference's rows reach its file out of order
            rb = deinterleave_reference_iop_rows(rb, 3 * 8 * 10 * 6).ravel()
        assert ra.shape == rb.shape and rel_l2(ra, rb) < 1e-9, name
    assert gzip.decompress(open(d + "fluid.0001.fluid3d.gz", "rb").read()) == \
        gzip.decompress(open(da + "fluid.0001.fluid3d.gz", "rb").read())
    for f in sorted(os.listdir(d)):
        if not f.endswith(".gz"):
            assert open(d + f, "rb").read() == open(da + f, "rb").read(), f


@pytest.mark.gpu
def test_postiop_and_iop_before_a_moving_step_and_without_cache():
    from cfs_plume_gb300.plume import BOX, Plume, PlumeError
    g = Plume(_abi.default_params(res=(12, 14, 10)))
    with pytest.raises(PlumeError):
        g.field("postIOP")
    with pytest.raises(PlumeError):
        g.iop()
    g.add_source(0)
    g.step()
    with pytest.raises(PlumeError):
        g.field("postIOP")
    box = BOX((0.5, 0.5, 0.5), (0.4, 0.4, 0.4), 4.0, 8.0)
    box.set_dt(0.1)
    g.step_moving_box(box)
    assert g.field("postIOP").shape == (3 * 12 * 14 * 10,)
    h = Plume(_abi.default_params(res=(12, 14, 10), cache_fields=0))
    h.step_moving_box(box)
    inside, _ = h.iop()
    assert inside.sum() > 0
    with pytest.raises(PlumeError):
        h.field("postIOP")
    bad = BOX((0.5, 0.5, 0.5), (0.4, 0.4, 0.4), 0.0, 8.0)  # zero period
    with pytest.raises(PlumeError):
        g.step_moving_box(bad)


@pytest.mark.gpu
def test_run_moving_timed_matches_step_loop_and_times_the_stomp():
    """plume_run_moving_timed (source, moving step, spin, translate per step)
    gives the same fields and box as the same loop through the single-step
    calls; with profiling on it times one stomp launch per step."""
    from cfs_plume_gb300.plume import Plume
    z = _fixture("box_open_14x12x16")
    p = _params_from(z)
    a, b = Plume(p), Plume(p)
    ba, bb = _gpu_box(z), _gpu_box(z)
    ms, st = a.run_moving_timed(ba, 0, 5)
    assert ms > 0 and len(st) == 5
    for s in range(5):
        b.add_source(s)
        b.step_moving_box(bb)
        bb.spin()
        bb.translate_center()
    assert bytes(memoryview(ba.state)) == bytes(memoryview(bb.state))
    for name in _abi.FIELDS + ["postIOP"]:
        assert np.array_equal(a.field(name), b.field(name)), name
    a.profile_sweeps(True)
    a.run_moving_timed(ba, 5, 3, stats=False)
    ms, n = a.stomp_times()
    a.profile_sweeps(False)
    assert n == 3 and ms > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32])
def test_stomp_mask_on_exact_box_faces(precision):
    """Cell centres exactly on the box faces (|q| = half, which BOX::inside
    counts as inside) and a box reaching past the domain, unrotated and then
    rotated: the GPU mask and last column equal the oracle's bit for bit."""
    from cfs_plume_gb300.plume import BOX, Plume
    res = (16, 16, 16)
    p = _abi.default_params(res=res, precision=precision, source=_abi.SRC_NONE, max_iters=0)
    # faces through the cell centres x = 4, 11 ((x + 0.5) / 16 = 0.28125, 0.71875)
    # and z = 1, 9 (0.09375, 0.59375), all exact in binary
    c, l = (0.5, 0.5, 0.34375), (0.4375, 0.25, 0.5)
    g = Plume(p)
    o = oracle.Oracle(p)
    bg = BOX(c, l, 0.8, 1.3)
    bg.set_dt(0.1)
    bo = oracle.box_init(c, l, 0.8, 1.3)
    bo.dt = 0.1
    for s in range(4):
        g.step_moving_box(bg)
        o.step_moving_box(bo)
        inside, vals = g.iop()
        assert np.array_equal(inside, _mask_numpy(res, bo))
        dims, ij, val = _iop_from_mask(res, inside, vals)
        odims, oij, oval = o.iop_entries()
        assert dims == odims and np.array_equal(ij, oij), s
        assert np.array_equal(val.view(np.uint64), oval.view(np.uint64)), s
        if s == 0:
            m = inside.reshape(16, 16, 16)
            assert m[:, :, 4].any() and m[:, :, 11].any() and m[1, :, :].any() and m[9, :, :].any()
            assert not m[:, :, 3].any() and not m[:, :, 12].any() and not m[10, :, :].any()
        bg.spin()
        bg.translate_center()
        oracle.box_spin(bo)
        oracle.box_translate(bo)
