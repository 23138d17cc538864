"""The snapshot SVD of svdOutOfCoreMultiple (include/plume_svd.h).

CPU: the numpy restatement (oracle/svd_oracle.py) against the reference's own
program (oracle/_ref/svd_ref, fixtures from tests/golden/make_golden.py) on the
six streams of a moving-box run.

GPU (through the C ABI and the stage binary), tolerances:
 * PCA values (S^2): |d| <= 1e-12 * S_0^2 (different dot-product orders in
   Gram-Schmidt, a different Jacobi method for the SVD of R: rounding-level);
 * U: the same kept count, each column equal up to its sign within 1e-10
   absolute (columns have unit norm) where the singular value is separated
   from its neighbours by a relative gap of 1e-6 (the fixtures: all);
 * file layouts byte-compatible with the reference's readers.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import svd_oracle as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = ["velocity.final", "velocity.preproject", "velocity.prediffuse", "velocity.preadvect",
         "pressure", "velocity.iop"]
TAGS = ["final", "preproject", "prediffuse", "preadvect", "pressure", "iop"]


def _fixture():
    return np.load(os.path.join(GOLDEN, "ref_svd_10x12x8.npz"))


def _matrix(z, tag):
    rows, cols = (int(v) for v in z["dims_" + tag][:2])
    return z["stream_" + tag].reshape(rows, cols).T


def _write_streams(z, d):
    for name, tag in zip(NAMES, TAGS):
        pre = os.path.join(d, name + ".matrix")
        z["dims_" + tag].astype("<i4").tofile(pre + ".dims")
        z["stream_" + tag].astype("<f8").tofile(pre + ".transpose")


def _close_u(U, ref, tol):
    assert U.shape == ref.shape
    Ua = S.align_signs(U, ref)
    return np.abs(Ua - ref).max() <= tol


# ------------------------------------------------------------------ CPU tests
@pytest.mark.parametrize("tag", TAGS)
def test_svd_oracle_matches_reference_program(tag):
    z = _fixture()
    pca, keep, U = S.svd_stream(_matrix(z, tag), float(z["threshold"]))
    ref_pca, ref_u = z["pca_" + tag], z["U_" + tag]
    assert np.abs(pca - ref_pca).max() <= 1e-12 * ref_pca[0]
    assert keep == ref_u.shape[1]
    assert _close_u(U, ref_u, 1e-10)


def test_reference_pca_files_are_empty_and_checks_are_tiny():
    """The reference's pca.*.vector copies a scratch file nothing writes, so it
    is empty; its projection check |c - U U^T c| is at rounding level."""
    z = _fixture()
    for tag in TAGS:
        assert int(z["pca_file_bytes_" + tag]) == 0
    assert z["verify_diffs"].size == 60 and z["verify_diffs"].max() < 1e-12


def test_svd_oracle_keep_rule():
    """Columns are kept until the first PCA ratio below the threshold."""
    assert S.kept_columns(np.array([4.0, 2.0, 1e-3, 1.0]), 1e-2) == 2
    assert S.kept_columns(np.array([4.0, 4.0]), 1.0) == 2


# ------------------------------------------------------------------ GPU tests
@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
def test_svd_stream_matches_reference(tmp_path, tag):
    from cfs_plume_gb300 import plume
    z = _fixture()
    snap, red, scr = str(tmp_path / "snap") + "/", str(tmp_path / "red") + "/", str(tmp_path / "scratch") + "/"
    for d in (snap, red, scr):
        os.makedirs(d)
    _write_streams(z, snap)
    name = NAMES[TAGS.index(tag)]
    # snapshot path one character longer than the reduced path: the reference's
    # name rule then gives "<stream>.matrix.singularValues.vector"
    snap2 = str(tmp_path / "snap_") + "/"
    os.rename(snap, snap2)
    info = plume.svd_stream(snap2 + name + ".matrix", red, scr, float(z["threshold"]),
                            red + "U." + tag + ".matrix", red + "pca." + tag + ".vector")
    ref_pca, ref_u = z["pca_" + tag], z["U_" + tag]
    assert info["kept"] == ref_u.shape[1] and info["cols"] == ref_pca.size
    U = S.read_u(red + "U." + tag + ".matrix")
    assert _close_u(U, ref_u, 1e-10)
    sv = S.read_vector(scr + name + ".matrix.singularValues.vector")
    assert np.abs(sv - ref_pca).max() <= 1e-12 * ref_pca[0]
    assert np.array_equal(S.read_vector(red + "pca." + tag + ".vector"), sv)
    d = plume.svd_verify(snap2 + name + ".matrix", red + "U." + tag + ".matrix", 10)
    assert d.max() < 1e-12


@pytest.mark.gpu
def test_svd_stage_binary(tmp_path):
    """bin/svdOutOfCoreMultiple with the reference's cfg keys on all six
    streams: the same U files (up to column signs) and checks."""
    from cfs_plume_gb300 import build
    build.build()
    z = _fixture()
    snap, red, scr = str(tmp_path / "snap_") + "/", str(tmp_path / "red") + "/", str(tmp_path / "scr") + "/"
    os.makedirs(snap)
    _write_streams(z, snap)
    cfg = tmp_path / "svd.cfg"
    cfg.write_text("snapshot path = %s\nreduced path = %s\nscratch path = %s\nsimulation snapshots = 12\n"
                   "reduced snapshots = 12\ndiscard threshold = 1e-9\niop = 1\n" % (snap, red, scr))
    exe = os.path.join(ROOT, "cfs_plume_gb300", "bin", "svdOutOfCoreMultiple")
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for tag in TAGS:
        assert _close_u(S.read_u(red + "U." + tag + ".matrix"), z["U_" + tag], 1e-10), tag
    diffs = [float(l.split(":")[1]) for l in r.stdout.splitlines() if l.strip().startswith("Diff")]
    assert len(diffs) == 60 and max(diffs) < 1e-12


def _decaying(n, m, seed, decay=0.7):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, m))
    Y = np.linalg.qr(rng.standard_normal((m, m)))[0]
    return (X * decay ** np.arange(m)) @ Y


@pytest.mark.gpu
@pytest.mark.parametrize("n,m,thr", [(40000, 150, 1e-9), (40000, 151, 1e-6), (3000, 1, 1e-9),
                                     (70001, 37, 1e-12)])
def test_svd_columns_vs_oracle(n, m, thr):
    """Random snapshots with a geometric spectrum (including an odd m, m = 1 and
    a row count that is not a multiple of the 2048-row block): PCA values,
    the kept count and U against the numpy restatement."""
    from cfs_plume_gb300 import plume
    A = _decaying(n, m, seed=n + m)
    pca, keep, U, info = plume.svd_columns(A, thr)
    opca, okeep, oU = S.svd_stream(A, thr)
    assert keep == okeep and info["kept"] == keep
    assert np.abs(pca - opca).max() <= 1e-12 * opca[0]
    # columns whose singular value is isolated by a relative gap of 1e-6
    s = np.sqrt(opca[:keep])
    gap = np.ones(keep)
    if keep > 1:
        rel = np.abs(np.diff(s)) / s[:-1]
        gap[:-1] = np.minimum(gap[:-1], rel)
        gap[1:] = np.minimum(gap[1:], rel)
    sel = gap > 1e-6
    Ua = S.align_signs(U, oU)
    err = np.abs(Ua - oU).max(axis=0)
    # a column's error scales with eps * s_0 / (s_k * gap)
    bound = 1e-10 * (s[0] / s) / np.maximum(gap, 1e-6)
    assert np.all(err[sel] <= np.maximum(bound[sel], 1e-10)), (err[sel].max(), info)
    assert np.abs(U.T @ U - np.eye(keep)).max() < 1e-8


@pytest.mark.gpu
def test_svd_columns_deterministic():
    from cfs_plume_gb300 import plume
    A = _decaying(30000, 64, seed=3)
    a = plume.svd_columns(A, 1e-9)
    b = plume.svd_columns(A, 1e-9)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_snapshots_equal_stream_files_and_their_svd(tmp_path, precision):
    """Rows kept in device memory (plume_snapshots) equal the stream files that
    plume_append_streams writes, for all six streams of a moving-box run, and
    their in-place SVD equals plume_svd_stream on those files."""
    from cfs_plume_gb300 import _abi, plume
    prec = _abi.PREC_FP64 if precision == "fp64" else _abi.PREC_FP32
    g = plume.Plume(_abi.default_params(res=(14, 16, 12), vorticity_eps=1.0, precision=prec))
    box = plume.BOX((0.5, 0.35, 0.5), (0.4, 0.3, 0.35), 2.0, 3.0)
    box.set_dt(0.1)
    snaps = {t: plume.Snapshots(g, t, 64) for t in TAGS}
    d = str(tmp_path / "snap_") + "/"
    os.makedirs(d)
    for s in range(10):
        g.add_source(s)
        g.step_moving_box(box)
        box.spin()
        box.translate_center()
        g.append_streams(d)
        for sn in snaps.values():
            sn.append()
    red, scr = str(tmp_path / "red") + "/", str(tmp_path / "scr") + "/"
    os.makedirs(red)
    os.makedirs(scr)
    for name, tag in zip(NAMES, TAGS):
        pre = d + name + ".matrix"
        A, rows, cols = S.read_stream(pre)
        held = snaps[tag].rows()
        assert held.shape == (rows, cols), tag
        assert np.array_equal(held, A.T), tag
        info = plume.svd_stream(pre, red, scr, 1e-9, red + "U." + tag + ".matrix")
        pca, kept, info2 = snaps[tag].svd(1e-9, u_path=red + "Ud." + tag + ".matrix")
        assert kept == info["kept"], tag
        assert np.array_equal(S.read_u(red + "U." + tag + ".matrix"), S.read_u(red + "Ud." + tag + ".matrix")), tag
        assert snaps[tag].dims()[0] == 0
    for sn in snaps.values():
        sn.close()
