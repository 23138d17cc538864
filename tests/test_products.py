"""The projected operators of the reduced model (plume_reduced_build_products,
include/plume_reduced.h) against the reference's own buildOutOfCoreMatrices:
the files that SUBSPACE_FLUID_3D_EIGEN's constructor (oracle/_ref/reduced_ref)
wrote for the bases of tests/golden/ref_reduced_exact_10x12x8.npz, under the
default walls and under mixed walls (ref_products_mixed_10x12x8.npz).

Tolerances (relative to the largest entry): the CPU restatement
(oracle/products_oracle.py) within 1e-12; the GPU build within 1e-12 for the
five projections (the reference sums over sparse rows in row order, the GPU
over 32-row chunks and splits) and 1e-10 for inverseProduct (the reference
inverts with Eigen's LU, the GPU by Gauss-Jordan elimination); the reduced
steps on the GPU-built operators within 1e-8 of the reference's run on its
own operators.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, os.path.dirname(HERE))

BASES = ["U.pressure.matrix", "U.preproject.matrix", "U.prediffuse.matrix", "U.final.matrix"]
PRODUCTS = ["projected.A", "projected.vtod", "damping.peeled", "projected.ptof", "projected.ptov",
            "inverseProduct"]
DEFAULT_BC = (1, 1, 1, 1, 0, 0)


def _matrix(raw):
    hdr = np.frombuffer(raw[:8].tobytes(), dtype="<i4")
    return np.frombuffer(raw[8:].tobytes(), dtype="<f8").reshape(int(hdr[0]), int(hdr[1]))


def _read(path):
    return _matrix(np.fromfile(path, dtype=np.uint8))


def _cases():
    z = np.load(os.path.join(GOLDEN, "ref_reduced_exact_10x12x8.npz"))
    m = np.load(os.path.join(GOLDEN, "ref_products_mixed_10x12x8.npz"))
    return {"default": (z, DEFAULT_BC, z), "mixed": (z, tuple(int(b) for b in m["bc"]), m)}


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# ------------------------------------------------------------------ CPU tests
@pytest.mark.parametrize("case", ["default", "mixed"])
def test_oracle_matches_reference_products(case):
    from oracle import products_oracle as po
    bases, bc, ref = _cases()[case]
    U = [_matrix(bases["file_" + f]) for f in BASES]
    got = po.products(tuple(int(v) for v in bases["res"]), bc, *U)
    for name in PRODUCTS:
        r = _matrix(ref["file_%s.matrix" % name])
        assert got[name].shape == r.shape, name
        assert _rel(got[name], r) < 1e-12, (name, _rel(got[name], r))


def test_mixed_walls_change_the_wall_dependent_operators():
    """The second fixture exercises other branches: projected.A and vtod
    depend on the walls, damping, ptof and ptov do not."""
    c = _cases()
    for name in PRODUCTS:
        a = _matrix(c["default"][2]["file_%s.matrix" % name])
        b = _matrix(c["mixed"][2]["file_%s.matrix" % name])
        if name in ("projected.A", "projected.vtod", "inverseProduct"):
            assert _rel(a, b) > 1e-3, name
        else:
            assert np.array_equal(a, b), name


def test_restated_operators_are_the_reference_stencils():
    """Structure of the restated sparse operators on a 6x7x5 grid: flat A and
    D are symmetric (so the reference's left^T M^T right equals
    left^T M right for them), D has 1 - w on its diagonal, V and G have the
    peeled shapes, and G maps a constant pressure to zero velocity."""
    from oracle import products_oracle as po
    res, bc = (6, 7, 5), DEFAULT_BC
    A = po.flat_a(res, bc).toarray()
    assert np.array_equal(A, A.T)
    D = po.damping(res).toarray()
    assert np.array_equal(D, D.T)
    assert np.allclose(np.diag(D), 0.1)
    V = po.velocity_to_divergence(res, bc, 1.0 / 7).toarray()
    G = po.pressure_to_velocity(res, 1.0 / 7).toarray()
    assert V.shape == (4 * 5 * 3, 3 * 4 * 5 * 3) and G.shape == (3 * 4 * 5 * 3, 4 * 5 * 3)
    # a constant pressure has no gradient
    assert np.abs(G @ np.ones(G.shape[1])).max() < 1e-12


# ------------------------------------------------------------------ GPU tests
def _plume(res, bc):
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    return Plume(_abi.default_params(res=res, bc=bc, vorticity_eps=1.0))


def _write(z, d, names):
    os.makedirs(d, exist_ok=True)
    for fn in names:
        z["file_" + fn].tofile(os.path.join(d, fn))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["default", "mixed"])
def test_gpu_build_matches_reference_products(tmp_path, case):
    from cfs_plume_gb300.plume import build_products
    bases, bc, ref = _cases()[case]
    d = str(tmp_path / "red") + "/"
    _write(bases, d, BASES)
    g = _plume(tuple(int(v) for v in bases["res"]), bc)
    info = build_products(g, d)
    U = [_matrix(bases["file_" + f]) for f in BASES]
    assert info["ranks"] == tuple(u.shape[1] for u in U)
    assert info["ms_device"] > 0 and info["gflop"] > 0
    for name in PRODUCTS:
        got = _read(d + name + ".matrix")
        r = _matrix(ref["file_%s.matrix" % name])
        assert got.shape == r.shape, name
        tol = 1e-10 if name == "inverseProduct" else 1e-12
        assert _rel(got, r) < tol, (name, _rel(got, r))


@pytest.mark.gpu
def test_reduced_model_from_bases_alone(tmp_path):
    """Only the bases and the cubature file under the reduced path: creating
    the model builds the projected operators (and the cubature cache), and 12
    reduced steps then track the reference's run on its own operators."""
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, ReducedModel
    z = np.load(os.path.join(GOLDEN, "ref_reduced_exact_10x12x8.npz"))
    d = str(tmp_path / "red") + "/"
    _write(z, d, BASES + ["U.preadvect.matrix", "cubature"])
    res = tuple(int(v) for v in z["res"])
    g = Plume(_abi.default_params(res=res, vorticity_eps=float(z["vorticity_eps"])))
    m = ReducedModel(g, d)
    for name in PRODUCTS:
        assert os.path.exists(d + name + ".matrix"), name
    for s in range(int(z["steps"])):
        g.add_source(s)
        m.step()
    assert _rel(m.qdot(), z["qdot"]) < 1e-8
    for name in ("velocity", "density", "heat"):
        f, r = g.field(name), z[name]
        err = np.linalg.norm(f - r) / np.linalg.norm(r)
        assert err < 1e-8, (name, err)


@pytest.mark.gpu
def test_stale_operators_are_rebuilt(tmp_path):
    """initOutOfCore: projected.ptof without a row per U.final column means
    the operators are stale, and all six are rebuilt."""
    from cfs_plume_gb300.plume import ReducedModel
    z = np.load(os.path.join(GOLDEN, "ref_reduced_exact_10x12x8.npz"))
    d = str(tmp_path / "red") + "/"
    _write(z, d, BASES + ["U.preadvect.matrix", "cubature"] + [p + ".matrix" for p in PRODUCTS])
    stale = np.zeros((3, 4))
    with open(d + "projected.ptof.matrix", "wb") as f:
        np.array(stale.shape, dtype="<i4").tofile(f)
        stale.tofile(f)
    g = _plume(tuple(int(v) for v in z["res"]), DEFAULT_BC)
    m = ReducedModel(g, d)
    got = _read(d + "projected.ptof.matrix")
    ref = _matrix(z["file_projected.ptof.matrix"])
    assert got.shape == ref.shape and _rel(got, ref) < 1e-12
    assert m.dims()["final"] == ref.shape[0]


@pytest.mark.gpu
def test_build_rejects_missing_bases_and_a_singular_pressure_matrix(tmp_path):
    from cfs_plume_gb300.plume import PlumeError, build_products
    z = np.load(os.path.join(GOLDEN, "ref_reduced_exact_10x12x8.npz"))
    res = tuple(int(v) for v in z["res"])
    d = str(tmp_path / "red") + "/"
    _write(z, d, BASES[1:])
    g = _plume(res, DEFAULT_BC)
    with pytest.raises(PlumeError):  # no U.pressure.matrix
        build_products(g, d)
    with pytest.raises(PlumeError):  # another grid
        _write(z, d, BASES)
        build_products(_plume((12, 12, 8), DEFAULT_BC), d)
    # a zero pressure column makes projected.A singular
    Up = _matrix(z["file_U.pressure.matrix"]).copy()
    Up[:, 3] = 0.0
    with open(d + "U.pressure.matrix", "wb") as f:
        np.array(Up.shape, dtype="<i4").tofile(f)
        Up.tofile(f)
    with pytest.raises(PlumeError, match="singular"):
        build_products(g, d)


@pytest.mark.gpu
@pytest.mark.parametrize("rank_p", [64, 120])
def test_gpu_build_matches_restatement_on_random_bases(tmp_path, rank_p):
    """Seeded random bases on the 10x12x8 grid under the mixed walls, against
    the scipy restatement: a pressure rank that the one-block elimination
    handles (64) and one above its shared-memory limit of 96 (120, one launch
    pair per pivot column)."""
    from oracle import products_oracle as po
    from cfs_plume_gb300.plume import build_products
    res, bc = (10, 12, 8), (0, 1, 1, 0, 1, 0)
    nint = 8 * 10 * 6
    rng = np.random.default_rng(rank_p)
    U = [rng.standard_normal((nint, rank_p)) / np.sqrt(nint)]
    U += [rng.standard_normal((3 * nint, r)) / np.sqrt(3 * nint) for r in (40, 33, 25)]
    d = str(tmp_path / "red") + "/"
    os.makedirs(d)
    for fn, M in zip(BASES, U):
        with open(d + fn, "wb") as f:
            np.array(M.shape, dtype="<i4").tofile(f)
            M.astype("<f8").tofile(f)
    info = build_products(_plume(res, bc), d)
    assert info["ranks"] == (rank_p, 40, 33, 25)
    want = po.products(res, bc, *U)
    for name in PRODUCTS:
        got = _read(d + name + ".matrix")
        assert got.shape == want[name].shape, name
        tol = 1e-10 if name == "inverseProduct" else 1e-12
        assert _rel(got, want[name]) < tol, (name, _rel(got, want[name]))


# ------------------------------------------------- the buildProducts binary
EXE = os.path.join(os.path.dirname(HERE), "cfs_plume_gb300", "bin", "buildProducts")


@pytest.fixture(scope="module")
def exe():
    from cfs_plume_gb300 import build
    build.build()
    assert os.path.exists(EXE)
    return EXE


def test_binary_usage_without_cfg(exe):
    import subprocess
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout


def test_binary_rejects_a_malformed_cfg_and_iop(exe, tmp_path):
    import subprocess
    bad = tmp_path / "bad.cfg"
    bad.write_text("xres = 10\nno equals sign here\n")
    r = subprocess.run([exe, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "Unable to parse" in r.stderr
    iop = tmp_path / "iop.cfg"
    iop.write_text("xRes = 10\nyRes = 12\nzRes = 8\niop = 1\nreduced path = %s/\n" % tmp_path)
    r = subprocess.run([exe, str(iop)], capture_output=True, text=True)
    assert r.returncode == 1 and "initOutOfCoreIOP" in r.stderr


@pytest.mark.gpu
def test_binary_builds_the_reference_operators(exe, tmp_path):
    """bin/buildProducts with the reference's cfg keys on the bases and
    cubature of the exact fixture: the six operators and the cubature cache
    written under `reduced path` are the reference's."""
    import subprocess
    z = np.load(os.path.join(GOLDEN, "ref_reduced_exact_10x12x8.npz"))
    d = str(tmp_path / "red") + "/"
    _write(z, d, BASES + ["U.preadvect.matrix", "cubature"])
    cfg = tmp_path / "products.cfg"
    cfg.write_text("xRes = 10\nyRes = 12\nzRes = 8\nreduced path = %s\nsnapshot path = %s/snap/\n"
                   "simulation snapshots = 12\n" % (d, tmp_path))
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for name in PRODUCTS:
        got = _read(d + name + ".matrix")
        ref = _matrix(z["file_%s.matrix" % name])
        tol = 1e-10 if name == "inverseProduct" else 1e-12
        assert got.shape == ref.shape and _rel(got, ref) < tol, name
    built = np.fromfile(d + "advection.cubature.cache", dtype=np.uint8)
    assert np.array_equal(built, z["file_advection.cubature.cache"])
