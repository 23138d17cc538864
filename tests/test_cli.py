"""The `fluid3D <cfg>` drop-in binary (projects/fluid3D/fluid3D.cpp:300-398):
command line, cfg parsing with the reference parser's rules, and on a GPU the
files it writes."""
import os
import subprocess

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import oracle
from tests.state_format import read_state

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "cfs_plume_gb300", "bin", "fluid3D")


@pytest.fixture(scope="module")
def exe():
    from cfs_plume_gb300 import build
    build.build()
    assert os.path.exists(EXE)
    return EXE


def test_usage_without_cfg(exe):
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout


def test_malformed_cfg_is_rejected(exe, tmp_path):
    cfg = tmp_path / "bad.cfg"
    cfg.write_text("xres = 16\nthis line has no equals sign\n")
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True)
    assert r.returncode == 1 and "Unable to parse" in r.stderr


def test_missing_cfg_is_reported(exe, tmp_path):
    r = subprocess.run([exe, str(tmp_path / "absent.cfg")], capture_output=True, text=True)
    assert r.returncode == 1 and "Failed to open" in r.stderr


@pytest.mark.gpu
def test_cli_run_matches_oracle(exe, tmp_path):
    """Two steps of a 12x14x10 plume with the reference's cfg keys: the state
    files and streams parse in the reference layout and hold the oracle's
    fields (FP64, reference stop test)."""
    snap = str(tmp_path) + "/snaps/"
    cfg = tmp_path / "plume.cfg"
    cfg.write_text("# comment line\nxRes = 12\nyres = 14\nZRES = 10\nvorticity = 1.5\n"
                   "snapshot path = %s\nsimulation snapshots = 2\n" % snap)
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    p = _abi.default_params(res=(12, 14, 10), vorticity_eps=1.5)
    o = oracle.Oracle(p)
    for s in range(2):
        o.add_source(s)
        o.step()
    s1 = read_state(snap + "fluid.0001.fluid3d.gz")
    for name in ("velocity", "density", "pressure", "preadvection", "cachedQuadratic"):
        ref = o.field(name)
        err = np.linalg.norm(s1[name] - ref) / max(np.linalg.norm(ref), 1e-300)
        assert err < 1e-9, (name, err)
    dims = np.fromfile(snap + "velocity.final.matrix.dims", dtype="<i4")
    assert tuple(dims) == (2, 3 * 10 * 12 * 8)


@pytest.mark.gpu
def test_cli_learned_warm_start(exe, tmp_path):
    """`warm start = learned` loads the committed network next to the binary
    and every solve still meets the configured stop test."""
    snap = str(tmp_path) + "/snaps/"
    cfg = tmp_path / "learned.cfg"
    cfg.write_text("xres = 32\nyres = 48\nzres = 32\nvorticity = 2\nbuoyancy = 1\nprecision = fp32\n"
                   "solver criterion = rel2\nsolver tolerance = 1e-6\nsource = box\nsource noise = 0.05\n"
                   "source box = 11 1 11 19 4 19\ntop = 1\nbottom = 1\n"
                   "warm start = learned\nsnapshot path = %s\nsimulation snapshots = 3\n"
                   "write streams = 0\n" % snap)
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Using learned warm start" in r.stdout
    rel = [float(line.split("relative two norm:")[1].split()[0])
           for line in r.stdout.splitlines() if "relative two norm:" in line]
    assert len(rel) == 3 and all(v <= 1e-6 for v in rel)
    assert os.path.exists(snap + "fluid.0002.fluid3d.gz")
