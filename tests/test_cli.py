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


def test_resume_from_a_missing_or_foreign_state_file_is_refused(exe, tmp_path):
    """`resume from` is checked on the host before any device work: a missing
    file, and a state file of another grid (the reference's own 8x10x6 file
    under a 12x14x10 cfg), end the run with status 1 and a message."""
    cfg = tmp_path / "resume.cfg"
    cfg.write_text("xRes = 12\nyRes = 14\nzRes = 10\nresume from = %s\nsnapshot path = %s/s/\n"
                   % (tmp_path / "absent.fluid3d.gz", tmp_path))
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True)
    assert r.returncode == 1 and "resume from" in r.stderr and "could not open" in r.stderr
    ref = os.path.join(ROOT, "tests", "golden", "ref_state_8x10x6", "fluid.0001.fluid3d.gz")
    cfg.write_text("xRes = 12\nyRes = 14\nzRes = 10\nresume from = %s\nsnapshot path = %s/s/\n"
                   % (ref, tmp_path))
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True)
    assert r.returncode == 1 and "8x10x6" in r.stderr


def test_step_log_lines_are_json(tmp_path):
    """The `log file` line format (plume_cli::step_json), compiled from the
    binary's own header into a tiny program: every stats field, non-finite
    numbers as null, one parseable JSON object per line."""
    import json
    src = tmp_path / "t.cpp"
    src.write_text(
        '#include "cli_config.h"\n#include <cmath>\n#include <cstdio>\n'
        'struct S { int iterations, converged, fallback, launches; double max_residual, rel_residual,'
        ' rhs_norm, ms_total, ms_solve, ms_forces, ms_vorticity, ms_advection, ms_damping, ms_divergence,'
        ' ms_guess, ms_gradient; };\n'
        'int main() { S a{93, 1, 0, 471, 8.5e-11, 9.75e-7, 3.25, 29.8125, 21.5, 0.25, 0.5, 0.5, 0.25, 0.125,'
        ' 0.0, 0.25};\n'
        '  S b{1000, 0, 1, 5, NAN, INFINITY, 0.0, 1.0, 0.5, 0, 0, 0, 0, 0, 0, 0};\n'
        '  std::printf("%s\\n%s\\n", plume_cli::step_json(7, a, 1e6, 4).c_str(),'
        ' plume_cli::step_json(8, b).c_str()); }\n')
    out = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "cfs_plume_gb300", "csrc"), str(src), "-o",
                    str(out)], check=True)
    lines = subprocess.run([str(out)], capture_output=True, text=True, check=True).stdout.splitlines()
    a, b = (json.loads(l) for l in lines)
    gbs = a.pop("gbs")
    assert a == {"step": 7, "iterations": 93, "converged": 1, "fallback": 0, "launches": 471,
                 "max_residual": 8.5e-11, "rel_residual": 9.75e-7, "rhs_norm": 3.25, "ms_total": 29.8125,
                 "ms_solve": 21.5, "ms_forces": 0.25, "ms_vorticity": 0.5, "ms_advection": 0.5,
                 "ms_damping": 0.25, "ms_divergence": 0.125, "ms_guess": 0.0, "ms_gradient": 0.25}
    # algorithmic bytes per interior cell (S = 4) x 1e6 cells / ms
    assert gbs["forces"] == pytest.approx(16 * 1e6 / 0.25e6)
    assert gbs["vorticity"] == pytest.approx(74 * 1e6 / 0.5e6)
    assert gbs["advection"] == pytest.approx(40 * 1e6 / 0.5e6)
    assert gbs["damping"] == pytest.approx(24 * 1e6 / 0.25e6)
    assert gbs["divergence"] == pytest.approx(21 * 1e6 / 0.125e6)
    assert gbs["solve"] == pytest.approx((30 + 93 * 75) * 1e6 / 21.5e6)
    assert gbs["gradient"] == pytest.approx(28 * 1e6 / 0.25e6)
    assert b["max_residual"] is None and b["rel_residual"] is None and b["step"] == 8 and b["fallback"] == 1
    assert "gbs" not in b


def test_state_header_reads_like_the_reference_file():
    """plume_state_read_header on the reference's own state files: the 10
    header ints and 7 doubles of FLUID_3D_MIC::readGz."""
    import ctypes as C
    from cfs_plume_gb300.plume import load_library
    lib = load_library()
    for rel in ("ref_state_8x10x6/fluid.0001.fluid3d.gz", "ref_moving_state_10x12x8/fluid.0001.fluid3d.gz"):
        path = os.path.join(ROOT, "tests", "golden", rel)
        ints = (C.c_int32 * 10)()
        dbls = (C.c_double * 7)()
        lib.plume_state_read_header.restype = C.c_int
        assert lib.plume_state_read_header(os.fsencode(path), ints, dbls) == 0
        ref = read_state(path)
        assert tuple(ints) == tuple(ref["header_ints"])
        assert tuple(dbls) == tuple(ref["header_doubles"])


@pytest.mark.gpu
def test_read_state_resumes_bit_exact(tmp_path):
    """plume_read_state (FLUID_3D_MIC::readGz into a handle) as a checkpoint:
    two FP64 steps, the state written, a new handle reads it and takes the
    third step; its fields equal those of three straight steps bit for bit,
    and the step count and time come back from the file."""
    from cfs_plume_gb300.plume import Plume
    p = _abi.default_params(res=(16, 20, 12), vorticity_eps=2.0)
    straight = Plume(p)
    for s in range(2):
        straight.add_source(s)
        straight.step()
    path = str(tmp_path / "fluid.0001.fluid3d.gz")
    straight.write_state(path)
    straight.add_source(2)
    straight.step()
    resumed = Plume(p)
    resumed.read_state(path)
    info = resumed.info()
    assert info["total_steps"] == 2
    resumed.add_source(2)
    resumed.step()
    for name in ("velocity", "density", "heat", "pressure", "divergence", "vorticity"):
        assert np.array_equal(resumed.field(name), straight.field(name)), name
    straight.close()
    resumed.close()


@pytest.mark.gpu
def test_cli_resume_from_continues_the_run(exe, tmp_path):
    """`resume from` in fluid3D: a run of 2 steps, then a second run resumed
    from its last state file for one more step, writes the same third state
    file as a straight 3-step run (FP64, reference stop test)."""
    base = "xRes = 12\nyRes = 14\nzRes = 10\nvorticity = 1.5\nwrite streams = 0\n"
    a, b = str(tmp_path) + "/a/", str(tmp_path) + "/b/"
    (tmp_path / "a.cfg").write_text(base + "snapshot path = %s\nsimulation snapshots = 3\n" % a)
    (tmp_path / "b1.cfg").write_text(base + "snapshot path = %s\nsimulation snapshots = 2\n" % b)
    (tmp_path / "b2.cfg").write_text(base + "snapshot path = %s\nsimulation snapshots = 3\n"
                                     "resume from = %sfluid.0001.fluid3d.gz\n" % (b, b))
    for c in ("a.cfg", "b1.cfg", "b2.cfg"):
        r = subprocess.run([exe, str(tmp_path / c)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, (c, r.stderr)
    assert "Resuming after step 2" in r.stdout
    sa, sb = read_state(a + "fluid.0002.fluid3d.gz"), read_state(b + "fluid.0002.fluid3d.gz")
    assert tuple(sa["header_ints"]) == tuple(sb["header_ints"])
    for name in _abi.FIELDS:
        assert np.array_equal(sa[name], sb[name]), name
