"""The files this build's fluid3D stage writes, read by the reference's own
compiled readers.

tests/golden/gpu_format_10x12x8/ holds what a GB300 wrote through the C ABI
(make_gpu_format_fixture.py): the state file of the last of 4 steps
(plume_write_state, the writeGz layout of FLUID_3D_MIC.cpp:1020-1110), the
six streams (plume_append_streams, appendStreams of 1329-1477) and every field
downloaded from the device.  Here, on the CPU:

 * the reference's FLUID_3D_MIC::readGz (FLUID_3D_MIC.cpp:1115-1246, compiled
   unmodified into oracle/_ref/fluid3d_ref) reads the state file and returns
   every field bit for bit as the device held it;
 * the reference's svdOutOfCoreMultiple (oracle/_ref/svd_ref, its own main)
   consumes the streams unchanged: its PCA values and bases equal those of the
   restated SVD (oracle/svd_oracle.py) of the rows, and those rows are the
   peeled fields of the device.

Skipped where the reference is not built (it needs the reference tree).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import svd_oracle as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FX = os.path.join(ROOT, "tests", "golden", "gpu_format_10x12x8")
REF = os.path.join(ROOT, "oracle", "_ref", "fluid3d_ref")
SVD_REF = os.path.join(ROOT, "oracle", "_ref", "svd_ref")
NAMES = ["velocity.final", "velocity.preproject", "velocity.prediffuse", "velocity.preadvect", "pressure"]
TAGS = ["final", "preproject", "prediffuse", "preadvect", "pressure"]


def _fields():
    return np.load(os.path.join(FX, "fields.npz"))


def _need(path):
    if not os.path.exists(path):
        pytest.skip("the reference is not built here (make -C oracle ref)")


def test_reference_readgz_reads_the_gpu_state_file(tmp_path):
    _need(REF)
    f = _fields()
    state = os.path.join(FX, "fluid.%04d.fluid3d.gz" % (int(f["steps"]) - 1))
    subprocess.run([REF, "readgz", state, str(tmp_path / "x")], check=True, capture_output=True)
    for name in _abi.FIELDS:
        got = np.fromfile(str(tmp_path / ("x.%s.f64" % name)))
        assert np.array_equal(got, f[name]), name


def _peel(a, res, ncomp):
    X, Y, Z = res
    v = a.reshape(Z, Y, X, ncomp)[1:-1, 1:-1, 1:-1]
    return v.reshape(-1)


def test_gpu_stream_rows_are_the_peeled_fields():
    """The last row of each stream is the peeled field of the last step, as
    appendStreams flattens it (x fastest, components interleaved); pressure
    holds two rows per step, pressure then divergence."""
    f = _fields()
    res = tuple(int(v) for v in f["res"])
    steps = int(f["steps"])
    last = {"final": f["velocity"], "preproject": f["preprojection"], "prediffuse": f["prediffusion"],
            "preadvect": f["preadvection"]}
    for name, tag in zip(NAMES, TAGS):
        A, rows, cols = S.read_stream(os.path.join(FX, name + ".matrix"))
        if tag == "pressure":
            assert rows == 2 * steps
            assert np.array_equal(A[:, -2], _peel(f["pressure"], res, 1))
            assert np.array_equal(A[:, -1], _peel(f["divergence"], res, 1))
        else:
            assert rows == steps and cols == 3 * (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
            assert np.array_equal(A[:, -1], _peel(last[tag], res, 3)), tag


def test_reference_svd_consumes_the_gpu_streams(tmp_path):
    _need(SVD_REF)
    f = _fields()
    steps = int(f["steps"])
    # the reference derives a file name by cutting the snapshot path's length
    # out of the reduced path; a snapshot path one character longer than the
    # reduced path yields "<stream>.matrix" (as in make_golden.py)
    snap, red, scr = str(tmp_path / "snap_") + "/", str(tmp_path / "red") + "/", str(tmp_path / "scratch") + "/"
    os.makedirs(snap)
    for fn in os.listdir(FX):
        if fn.endswith(".dims") or fn.endswith(".transpose"):
            shutil.copy(os.path.join(FX, fn), snap)
    cfg = tmp_path / "svd.cfg"
    cfg.write_text("snapshot path = %s\nreduced path = %s\nscratch path = %s\nsimulation snapshots = %d\n"
                   "reduced snapshots = %d\ndiscard threshold = 1e-9\n" % (snap, red, scr, steps, steps))
    subprocess.run([SVD_REF, str(cfg)], check=True, capture_output=True)
    for name, tag in zip(NAMES, TAGS):
        A, _, _ = S.read_stream(os.path.join(FX, name + ".matrix"))
        pca, keep, U = S.svd_stream(A, 1e-9)
        u = red + "U." + tag + ".matrix"
        hdr = np.fromfile(u, dtype="<i4", count=2)
        ref_u = np.fromfile(u, dtype="<f8", offset=8).reshape(int(hdr[0]), int(hdr[1]))
        sv = scr + name + ".matrix.singularValues.vector"
        nsv = int(np.fromfile(sv, dtype="<i4", count=1)[0])
        ref_pca = np.fromfile(sv, dtype="<f8", offset=4, count=nsv)
        assert ref_u.shape[1] == keep, tag
        assert np.abs(pca - ref_pca).max() <= 1e-12 * ref_pca[0], tag
        assert np.abs(S.align_signs(U, ref_u) - ref_u).max() <= 1e-9, tag
