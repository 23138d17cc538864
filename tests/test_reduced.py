"""The reduced step (include/plume_reduced.h) against the reference's own
SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam (oracle/_ref/reduced_ref,
fixtures from tests/golden/make_golden.py): bases that the reference's
svdOutOfCoreMultiple built from a 12-step 10x12x8 plume, the projected
operators its constructor built, and two cubature schemes (every interior cell
with weight 1, which makes the reduced advection an exact Galerkin projection;
40 seeded cells with seeded weights).

On the host: the ground-truth comparison that ends the reference's step
(diffGroundTruth), through plume_state_read_field and plume_peeled_errors,
reproduces the reference's recorded errors within 1e-12.

Tolerances: FP64 fields after 12 reduced steps within 1e-8 relative L2 of the
reference's (the reduced products sum in a different order: Eigen's GEMV and
block products against warp-level FMA reductions); the cubature cache built
here byte-identical to the reference's; FP32 fields within 1e-3.
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["exact_10x12x8", "sparse_10x12x8"]
# every file of a built model, so that the steps run on the reference's own
# projected operators (tests/test_products.py covers the GPU-built ones)
FILES = ["U.preadvect.matrix", "U.final.matrix", "U.prediffuse.matrix", "U.preproject.matrix",
         "U.pressure.matrix", "damping.peeled.matrix", "projected.ptof.matrix", "projected.A.matrix",
         "projected.vtod.matrix", "projected.ptov.matrix", "inverseProduct.matrix", "cubature",
         "advection.cubature.cache"]


def _fixture(case):
    return np.load(os.path.join(GOLDEN, "ref_reduced_%s.npz" % case))


def _matrix(raw):
    hdr = np.frombuffer(raw[:8].tobytes(), dtype="<i4")
    return np.frombuffer(raw[8:].tobytes(), dtype="<f8").reshape(int(hdr[0]), int(hdr[1]))


def _write_model(z, d, with_cache=True):
    os.makedirs(d, exist_ok=True)
    for fn in FILES:
        if fn == "advection.cubature.cache" and not with_cache:
            continue
        z["file_" + fn].tofile(os.path.join(d, fn))


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


# ------------------------------------------------------------------ CPU tests
@pytest.mark.parametrize("case", CASES)
def test_reference_cubature_cache_layout(case):
    """advection.cubature.cache = for each cubature cell its 3 rows of
    U.preadvect, then weight x its 3 rows of U.prediffuse transposed
    (SUBSPACE_FLUID_3D_EIGEN.cpp:1256-1299), each as EIGEN::write."""
    z = _fixture(case)
    raw = z["file_cubature"].tobytes()
    n = int(np.frombuffer(raw[:4], dtype="<i4")[0])
    cells = np.frombuffer(raw[4:4 + 4 * n], dtype="<i4")
    weights = np.frombuffer(raw[4 + 4 * n:4 + 12 * n], dtype="<f8")
    Upa = _matrix(z["file_U.preadvect.matrix"])
    Upd = _matrix(z["file_U.prediffuse.matrix"])
    cache = z["file_advection.cubature.cache"].tobytes()
    off = 0
    for x in range(n):
        r, c = np.frombuffer(cache[off:off + 8], dtype="<i4")
        m = np.frombuffer(cache[off + 8:off + 8 + 8 * r * c], dtype="<f8").reshape(r, c)
        assert np.array_equal(m, Upa[3 * cells[x]:3 * cells[x] + 3])
        off += 8 + 8 * r * c
    for x in range(n):
        r, c = np.frombuffer(cache[off:off + 8], dtype="<i4")
        m = np.frombuffer(cache[off + 8:off + 8 + 8 * r * c], dtype="<f8").reshape(r, c)
        assert np.array_equal(m, weights[x] * Upd[3 * cells[x]:3 * cells[x] + 3].T)
        off += 8 + 8 * r * c
    assert off == len(cache)


@pytest.mark.parametrize("case", CASES)
def test_oracle_restatement_matches_the_reference(tmp_path, case):
    """oracle/reduced_oracle.py (the C oracle's full-space prestep and the
    numpy reduced part) against the reference's own 12-step run: density and
    heat identical, velocity and q within 1e-12 (the reduced products sum in
    another order than Eigen's)."""
    from cfs_plume_gb300 import _abi
    from oracle import reduced_oracle
    z = _fixture(case)
    d = str(tmp_path / "red") + "/"
    _write_model(z, d)
    p = _abi.default_params(res=tuple(int(v) for v in z["res"]), vorticity_eps=float(z["vorticity_eps"]))
    o, q = reduced_oracle.run(p, d, int(z["steps"]))
    assert np.array_equal(o.field("density"), z["density"])
    assert np.array_equal(o.field("heat"), z["heat"])
    assert rel_l2(o.field("velocity"), z["velocity"]) < 1e-12
    assert rel_l2(q, z["qdot"]) < 1e-12


def test_oracle_restatement_matches_the_reference_under_mixed_walls(tmp_path):
    """The same under mixed walls (front, back, left, right, top, bottom =
    0 1 1 0 1 0): the reference's constructor built the operators for those
    walls, and its prestep takes the other face branches."""
    from cfs_plume_gb300 import _abi
    from oracle import reduced_oracle
    z = _fixture("exact_10x12x8")
    m = np.load(os.path.join(GOLDEN, "ref_products_mixed_10x12x8.npz"))
    d = str(tmp_path / "red") + "/"
    os.makedirs(d)
    for fn in ("U.preadvect.matrix", "U.final.matrix", "U.prediffuse.matrix", "cubature"):
        z["file_" + fn].tofile(d + fn)
    for fn in ("damping.peeled.matrix", "projected.ptof.matrix", "inverseProduct.matrix"):
        m["file_" + fn].tofile(d + fn)
    p = _abi.default_params(res=tuple(int(v) for v in m["res"]), bc=tuple(int(b) for b in m["bc"]),
                            vorticity_eps=float(m["vorticity_eps"]))
    o, q = reduced_oracle.run(p, d, int(m["steps"]))
    assert np.array_equal(o.field("density"), m["density"])
    assert np.array_equal(o.field("heat"), m["heat"])
    assert rel_l2(o.field("velocity"), m["velocity"]) < 1e-12
    assert rel_l2(q, m["qdot"]) < 1e-12


def test_exact_cubature_tracks_the_full_rank_run():
    """With every cell as a cubature point the reference's reduced run stays
    within 1e-4 (velocity) and 1e-7 (density) of the full-rank run."""
    e = _fixture("exact_10x12x8")["errors"]
    assert e[:, 1].max() < 1e-4 and e[:, 3].max() < 1e-7


@pytest.mark.parametrize("case", CASES)
def test_ground_truth_errors_match_the_reference(tmp_path, case):
    """diffGroundTruth on the host: the reference's last reduced fields
    against the full-rank state file of frame 11 (read back by
    plume_state_read_field), through plume_peeled_errors, give the
    reference's last recorded errors."""
    from cfs_plume_gb300.plume import peeled_errors, read_state_field
    z = _fixture(case)
    path = str(tmp_path / "fluid.0011.fluid3d.gz")
    z["truth_last"].tofile(path)
    tv, res = read_state_field(path, "velocity")
    td, _ = read_state_field(path, "density")
    assert res == tuple(int(v) for v in z["res"])
    err = peeled_errors(res, z["velocity"], z["density"], tv, td)
    ref = z["errors"][-1]
    assert np.allclose(err, ref, rtol=1e-12, atol=0), (err, ref)


def test_state_reader_follows_concatenated_gzip_members(tmp_path):
    """The state file cut into several gzip members (as the parallel writer
    emits it) reads back field for field like the single-member original."""
    import gzip
    from cfs_plume_gb300.plume import read_state_field
    z = _fixture("exact_10x12x8")
    one = str(tmp_path / "one.fluid3d.gz")
    z["truth_last"].tofile(one)
    raw = gzip.decompress(z["truth_last"].tobytes())
    many = str(tmp_path / "many.fluid3d.gz")
    with open(many, "wb") as f:
        for k in range(0, len(raw), 7001):
            f.write(gzip.compress(raw[k:k + 7001], compresslevel=1))
    for name in ("density", "velocity", "pressure", "prevorticity"):
        a, _ = read_state_field(one, name)
        b, _ = read_state_field(many, name)
        assert np.array_equal(a, b), name


def test_state_reader_reports_missing_and_mismatched_requests(tmp_path):
    from cfs_plume_gb300.plume import PlumeError, load_library, read_state_field
    with pytest.raises(PlumeError):
        read_state_field(str(tmp_path / "absent.fluid3d"), "density")
    z = _fixture("exact_10x12x8")
    path = str(tmp_path / "fluid.0011.fluid3d.gz")
    z["truth_last"].tofile(path)
    with pytest.raises(PlumeError, match="holds 0 values"):  # no moving-box step wrote postIOP
        read_state_field(path, "postIOP")
    lib = load_library()
    buf = np.empty(10)
    assert lib.plume_state_read_field(os.fsencode(path), 0, buf.ctypes.data, buf.size, None) != 0
    cut = str(tmp_path / "cut.fluid3d.gz")
    import gzip
    raw = gzip.decompress(z["truth_last"].tobytes())
    with open(cut, "wb") as f:
        f.write(gzip.compress(raw[:5000]))
    with pytest.raises(PlumeError, match="truncated"):
        read_state_field(cut, "velocity")


# ------------------------------------------------------------------ GPU tests
def _run(z, d, precision):
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, ReducedModel
    res = tuple(int(v) for v in z["res"])
    g = Plume(_abi.default_params(res=res, vorticity_eps=float(z["vorticity_eps"]), precision=precision))
    m = ReducedModel(g, d)
    for s in range(int(z["steps"])):
        g.add_source(s)
        st = m.step()
        assert st.launches > 0
    return g, m


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_reduced_step_matches_reference_fp64(tmp_path, case):
    from cfs_plume_gb300 import _abi
    z = _fixture(case)
    d = str(tmp_path / "red") + "/"
    # the exact case builds the cubature cache here; the sparse one reads it
    _write_model(z, d, with_cache=(case != "exact_10x12x8"))
    g, m = _run(z, d, _abi.PREC_FP64)
    if case == "exact_10x12x8":
        built = np.fromfile(d + "advection.cubature.cache", dtype=np.uint8)
        assert np.array_equal(built, z["file_advection.cubature.cache"])
    dims = m.dims()
    assert dims["final"] == z["qdot"].size
    assert rel_l2(m.qdot(), z["qdot"]) < 1e-8
    for name in ("velocity", "density", "heat"):
        err = rel_l2(g.field(name), z[name])
        assert err < 1e-8, "%s rel L2 %.3e" % (name, err)


@pytest.mark.gpu
def test_reduced_step_fp32(tmp_path):
    from cfs_plume_gb300 import _abi
    z = _fixture("exact_10x12x8")
    d = str(tmp_path / "red") + "/"
    _write_model(z, d)
    g, m = _run(z, d, _abi.PREC_FP32)
    for name in ("velocity", "density", "heat"):
        err = rel_l2(g.field(name), z[name])
        assert err < 1e-3, "%s rel L2 %.3e" % (name, err)


@pytest.mark.gpu
def test_reduced_model_rejects_mismatched_files(tmp_path):
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, PlumeError, ReducedModel
    z = _fixture("exact_10x12x8")
    d = str(tmp_path / "red") + "/"
    _write_model(z, d)
    with pytest.raises(PlumeError):  # another grid
        ReducedModel(Plume(_abi.default_params(res=(12, 12, 8))), d)
    # an operator missing and no pressure basis to rebuild it from
    os.remove(d + "inverseProduct.matrix")
    os.remove(d + "U.pressure.matrix")
    with pytest.raises(PlumeError):
        ReducedModel(Plume(_abi.default_params(res=(10, 12, 8))), d)


# ------------------------------------------------------ the reduced3D binary
RED_EXE = os.path.join(os.path.dirname(GOLDEN), "..", "cfs_plume_gb300", "bin", "reduced3D")


def test_reduced3d_binary_command_line(tmp_path):
    """bin/reduced3D: the reference's usage line, the cfg parser's errors, and
    the refusal of the IOP model, all before any device work."""
    import subprocess
    from cfs_plume_gb300 import build
    build.build()
    exe = os.path.abspath(RED_EXE)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout
    bad = tmp_path / "bad.cfg"
    bad.write_text("xres = 10\nno equals sign\n")
    r = subprocess.run([exe, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "Unable to parse" in r.stderr
    iop = tmp_path / "iop.cfg"
    iop.write_text("xRes = 10\nyRes = 12\nzRes = 8\niop = 1\n")
    r = subprocess.run([exe, str(iop)], capture_output=True, text=True)
    assert r.returncode == 1 and "initOutOfCoreIOP" in r.stderr


def _full_rank_truth(z, d):
    """The full-rank FP64 run of the fixture's plume on the GPU, its state
    file written after every step (fluid.%04i.fluid3d.gz, as fluid3D writes
    them): the ground truth diffGroundTruth reads."""
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    res = tuple(int(v) for v in z["res"])
    g = Plume(_abi.default_params(res=res, vorticity_eps=float(z["vorticity_eps"])))
    os.makedirs(d, exist_ok=True)
    for s in range(int(z["steps"])):
        g.add_source(s)
        g.step()
        g.write_state(os.path.join(d, "fluid.%04d.fluid3d.gz" % s))
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_ground_truth_errors_on_gpu_state_files(tmp_path, case):
    """The reduced step's ground-truth comparison (diffGroundTruth,
    SUBSPACE_FLUID_3D_EIGEN.cpp:804-835) on the GPU against state files this
    build's FP64 full-rank run wrote: every step's four errors agree with
    those the reference recorded against its own full-rank files (both runs
    and both reduced models agree to 1e-8, so the errors to 1e-3 relative)."""
    from cfs_plume_gb300 import _abi
    z = _fixture(case)
    d = str(tmp_path / "red") + "/"
    truth = str(tmp_path / "truth") + "/"
    _write_model(z, d)
    _full_rank_truth(z, truth)
    from cfs_plume_gb300.plume import Plume, ReducedModel
    res = tuple(int(v) for v in z["res"])
    g = Plume(_abi.default_params(res=res, vorticity_eps=float(z["vorticity_eps"])))
    m = ReducedModel(g, d)
    m.set_ground_truth(truth)
    for s in range(int(z["steps"])):
        g.add_source(s)
        m.step()
    e = m.errors()
    assert e.shape == z["errors"].shape
    np.testing.assert_allclose(e, z["errors"], rtol=1e-3, atol=1e-12)
    m.close()
    g.close()


@pytest.mark.gpu
def test_reduced3d_binary_runs_the_reference_model(tmp_path):
    """bin/reduced3D on the reference's sparse-cubature model with the
    reference's cfg keys, against this build's full-rank state files: it
    prints the reference's error vectors (every 10 steps and at the end) and
    the last ones equal the reference's recorded errors to 1e-3 relative."""
    import subprocess
    from cfs_plume_gb300 import build
    build.build()
    z = _fixture("sparse_10x12x8")
    d = str(tmp_path / "red") + "/"
    truth = str(tmp_path / "truth") + "/"
    _write_model(z, d)
    _full_rank_truth(z, truth)
    cfg = tmp_path / "reduced.cfg"
    cfg.write_text("xRes = 10\nyRes = 12\nzRes = 8\nvorticity = %r\nreduced path = %s\nsnapshot path = %s\n"
                   "simulation snapshots = %d\n" % (float(z["vorticity_eps"]), d, truth, int(z["steps"])))
    r = subprocess.run([os.path.abspath(RED_EXE), str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    vals = {}
    for line in r.stdout.splitlines():
        for k in ("velocityAbs", "velocityRelative", "densityAbs", "densityRelative"):
            if line.strip().startswith(k + " = ["):
                vals[k] = [float(v) for v in line.split("[")[1].split("]")[0].split()]
    last = [vals[k][-1] for k in ("velocityAbs", "velocityRelative", "densityAbs", "densityRelative")]
    assert len(vals["velocityAbs"]) == int(z["steps"])
    np.testing.assert_allclose(last, z["errors"][-1], rtol=1e-3, atol=1e-12)
