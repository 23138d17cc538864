"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs oracle/_ref/fluid3d_ref -- the reference's own FLUID_3D_MIC.cpp, compiled
unmodified by `make -C oracle ref` (headless driver in oracle/ref/) -- on small
configurations and stores what it produced:

  ref_<case>.npz        every state field after the last step (read back with
                        the reference's own FLUID_3D_MIC::readGz) and the PCG
                        iteration count of every step;
  ref_cfg1_sampled.npz  the 48x64x48 plume (box source, closed box, FP64,
                        reference criterion 1e-10), all 100 steps of its
                        configuration: iteration counts, per-field sums / L2
                        norms and every 97th value;
  ref_state_8x10x6/     the reference's own state file (writeGz, gzip level 1)
                        and appendStreams output after 2 steps, as format
                        fixtures;
  ref_moving_<case>.npz the moving-box step (stepWithMovingObstacle with the
                        BOX spun and translated after every step): every
                        state field, postIOP and the obstacle matrix's
                        (row, col, value) entries after the last step;
  ref_moving_state_10x12x8/  the reference's state file and streams of a
                        moving-box run, as format fixtures;
  ref_svd_10x12x8.npz   the reference's svdOutOfCoreMultiple (oracle/_ref/svd_ref,
                        its own main) on the six streams of a 12-step moving-box
                        run: the input streams, every U.*.matrix and every
                        singular-value vector;
  ref_reduced_<case>.npz  the reference's reduced step (oracle/_ref/reduced_ref:
                        SUBSPACE_FLUID_3D_EIGEN, stepReorderedCubatureStam) on
                        bases that svd_ref built from a 12-step plume: the
                        reduced-path files it read or wrote (bases, projected
                        operators, cubature, cubature cache) and the fields,
                        reduced coordinates and ground-truth errors after 12
                        reduced steps, and the full-rank state file of the last
                        frame that the last error compares against;
  ref_products_mixed_10x12x8.npz  the projected operators that the reference's
                        constructor (buildOutOfCoreMatrices) builds from the
                        same bases under mixed walls, and the fields and reduced
                        coordinates after 12 reduced steps under those walls.

Needs the reference built by `make -C oracle ref REF=<reference tree>` and
writes nothing outside tests/golden/.
Usage: python tests/golden/make_golden.py [plume|cfg1|moving|svd|reduced]   (default: all)
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cfs_plume_gb300 import _abi  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "fluid3d_ref")
SVD_REF = os.path.join(ROOT, "oracle", "_ref", "svd_ref")
SVD_STREAMS = ["velocity.final", "velocity.preproject", "velocity.prediffuse", "velocity.preadvect",
               "pressure", "velocity.iop"]
SVD_TAGS = ["final", "preproject", "prediffuse", "preadvect", "pressure", "iop"]

# name -> (params kwargs, steps, reference source mode)
CASES = {
    "default_16x20x12": (dict(res=(16, 20, 12)), 6, "column"),
    "vort2_16x20x12": (dict(res=(16, 20, 12), vorticity_eps=2.0), 6, "column"),
    "closed_box_17x23x13": (dict(res=(17, 23, 13), bc=(1, 1, 1, 1, 1, 1), vorticity_eps=1.0,
                                 buoyancy=1.0, source=_abi.SRC_BOX, box_lo=(6, 2, 4),
                                 box_hi=(11, 6, 9), source_noise=0.05, seed=7), 6, "box"),
    "mixed_bc_16x20x12": (dict(res=(16, 20, 12), bc=(0, 1, 0, 1, 0, 1), vorticity_eps=0.5), 6,
                          "column"),
    "open_box_20x16x18": (dict(res=(20, 16, 18), bc=(0, 0, 0, 0, 0, 0), vorticity_eps=1.5,
                               buoyancy=0.5, source=_abi.SRC_BOX, box_lo=(7, 1, 7),
                               box_hi=(13, 4, 11), source_noise=0.05, seed=11), 5, "box"),
}


def ref_args(p, steps, src, out):
    a = [REF, "run", "res=%d,%d,%d" % tuple(p.res), "bc=" + ",".join(str(b) for b in p.bc),
         "vorticity=%r" % p.vorticity_eps, "steps=%d" % steps, "out=%s/" % out, "dump=1",
         "source=" + src]
    if src == "box":
        a += ["box=%d,%d,%d,%d,%d,%d" % (tuple(p.box_lo) + tuple(p.box_hi)),
              "noise=%r" % p.source_noise, "seed=%d" % p.seed]
    if p.buoyancy != _abi.BUOYANCY_REF:
        a += ["buoyancy=%r" % p.buoyancy]
    return a


def run_ref(p, steps, src, extra=()):
    d = tempfile.mkdtemp(prefix="plume_golden_")
    r = subprocess.run(ref_args(p, steps, src, d) + list(extra), capture_output=True, text=True,
                       check=True)
    iters = [int(l.split()[0]) for l in r.stdout.splitlines() if "iterations converged" in l]
    subprocess.run([REF, "readgz", d + "/final.fluid3d.gz", d + "/x"], check=True,
                   capture_output=True)
    fields = {n: np.fromfile(d + "/x.%s.f64" % n) for n in _abi.FIELDS}
    fields["obstacles"] = np.fromfile(d + "/x.obstacles.u8", dtype=np.uint8)
    if os.path.exists(d + "/x.postIOP.f64"):
        fields["postIOP"] = np.fromfile(d + "/x.postIOP.f64")
        fields["iop_dims"] = np.fromfile(d + "/x.iop_dims.i32", dtype=np.int32)
        fields["iop_ij"] = np.fromfile(d + "/x.iop_ij.i32", dtype=np.int32).reshape(-1, 2)
        fields["iop_val"] = np.fromfile(d + "/x.iop_val.f64")
    return d, iters, fields


# name -> (params kwargs, steps, source, box center, box lengths, period,
#          translation period, setInitialVelocity first)
MOVING = {
    "box_16x20x12": (dict(res=(16, 20, 12), vorticity_eps=1.0), 4, "column",
                     (0.5, 0.4, 0.5), (0.3, 0.2, 0.4), 4.0, 8.0, True),
    # fast spin and sway: theta and phi wrap past 2 pi; open faces; the box
    # reaches out of the domain
    "box_open_14x12x16": (dict(res=(14, 12, 16), bc=(0, 0, 0, 0, 0, 0), vorticity_eps=0.5,
                               source=_abi.SRC_BOX, box_lo=(5, 1, 6), box_hi=(9, 3, 10),
                               source_noise=0.05, seed=3), 8, "box",
                          (0.85, 0.5, 0.45), (0.5, 0.3, 0.25), 0.45, 0.35, False),
}


def moving_args(c, l, period, tperiod, initvel):
    return ["moving=1", "boxc=%r,%r,%r" % tuple(c), "boxl=%r,%r,%r" % tuple(l),
            "period=%r" % period, "tperiod=%r" % tperiod, "initvel=%d" % int(initvel)]


def params_record(p):
    return dict(res=np.array(p.res), bc=np.array(p.bc), buoyancy=p.buoyancy,
                vorticity_eps=p.vorticity_eps, source=p.source, box_lo=np.array(p.box_lo),
                box_hi=np.array(p.box_hi), source_noise=p.source_noise, seed=p.seed)


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -C oracle ref")
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("all", "plume"):
        plume_fixtures()
    if what in ("all", "plume", "cfg1"):
        cfg1_fixture()
    if what in ("all", "moving"):
        moving_fixtures()
    if what in ("all", "svd"):
        svd_fixtures()
    if what in ("all", "reduced"):
        reduced_fixtures()


RED_REF = os.path.join(ROOT, "oracle", "_ref", "reduced_ref")
RED_FILES = ["U.preadvect.matrix", "U.final.matrix", "U.prediffuse.matrix", "U.preproject.matrix",
             "U.pressure.matrix", "damping.peeled.matrix", "projected.ptof.matrix", "projected.A.matrix",
             "projected.vtod.matrix", "projected.ptov.matrix", "inverseProduct.matrix", "cubature",
             "advection.cubature.cache"]
PRODUCT_FILES = ["projected.A.matrix", "projected.vtod.matrix", "damping.peeled.matrix",
                 "projected.ptof.matrix", "projected.ptov.matrix", "inverseProduct.matrix"]
# walls (front, back, left, right, top, bottom) of the second operator build:
# Neumann on the x-high, z-low and y-low faces, so that every branch of
# computeVelocityToDivergence and every wall pattern of buildFlatA is taken
MIXED_BC = (0, 1, 1, 0, 1, 0)


def reduced_fixtures():
    res, steps = (10, 12, 8), 12
    nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
    base = tempfile.mkdtemp(prefix="plume_golden_")
    snap, red0, scr = base + "/snap_/", base + "/red/", base + "/scratch/"
    os.makedirs(snap)
    p = _abi.default_params(res=res, vorticity_eps=1.0)
    # the full-rank run: streams for the bases, state files as ground truth
    subprocess.run(ref_args(p, steps, "column", snap) + ["streams=1", "gz=1"], check=True,
                   capture_output=True)
    cfg = base + "/svd.cfg"
    with open(cfg, "w") as f:
        f.write("snapshot path = %s\nreduced path = %s\nscratch path = %s\nsimulation snapshots = %d\n"
                "reduced snapshots = %d\ndiscard threshold = 1e-9\n" % (snap, red0, scr, steps, steps))
    subprocess.run([SVD_REF, cfg], check=True, capture_output=True)
    rng = np.random.default_rng(3)
    sparse = np.sort(rng.choice(nint, 40, replace=False)).astype("<i4")
    cases = {"exact_10x12x8": (np.arange(nint, dtype="<i4"), np.ones(nint)),
             "sparse_10x12x8": (sparse, (nint / 40.0) * rng.uniform(0.5, 1.5, 40))}
    for name, (cells, weights) in cases.items():
        red = base + "/red_" + name + "/"
        shutil.copytree(red0, red)
        with open(red + "cubature", "wb") as f:
            np.array([cells.size], dtype="<i4").tofile(f)
            cells.astype("<i4").tofile(f)
            np.asarray(weights, dtype="<f8").tofile(f)
        out = base + "/out_" + name
        subprocess.run([RED_REF, "res=%d,%d,%d" % res, "vorticity=1.0", "reduced=" + red, "truth=" + snap,
                        "steps=%d" % steps, "out=" + out], check=True, capture_output=True)
        rec = {"res": np.array(res), "steps": steps, "vorticity_eps": 1.0}
        for fn in RED_FILES:
            rec["file_" + fn] = np.fromfile(red + fn, dtype=np.uint8)
        for k in ("velocity", "density", "heat", "qdot"):
            rec[k] = np.fromfile(out + "." + k + ".f64")
        rec["errors"] = np.fromfile(out + ".errors.f64").reshape(-1, 4)
        # the full-rank state file of the last frame (diffGroundTruth's input)
        rec["truth_last"] = np.fromfile(snap + "fluid.%04d.fluid3d.gz" % (steps - 1), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, "ref_reduced_%s.npz" % name), **rec)
        print("reduced", name, "qdot", rec["qdot"].size, "errors (last)", rec["errors"][-1])
    # the projected operators of the same bases under other walls: the
    # reference's constructor builds them (buildOutOfCoreMatrices), no steps
    red = base + "/red_mixed/"
    shutil.copytree(red0, red)
    shutil.copy(base + "/red_exact_10x12x8/cubature", red + "cubature")
    out = base + "/out_mixed"
    subprocess.run([RED_REF, "res=%d,%d,%d" % res, "bc=" + ",".join(str(b) for b in MIXED_BC),
                    "vorticity=1.0", "reduced=" + red, "truth=" + snap, "steps=%d" % steps, "out=" + out],
                   check=True, capture_output=True)
    rec = {"res": np.array(res), "bc": np.array(MIXED_BC), "steps": steps, "vorticity_eps": 1.0}
    for fn in PRODUCT_FILES:
        rec["file_" + fn] = np.fromfile(red + fn, dtype=np.uint8)
    # the reduced steps under these walls (the bases are the default-wall run's)
    for k in ("velocity", "density", "heat", "qdot"):
        rec[k] = np.fromfile(out + "." + k + ".f64")
    np.savez_compressed(os.path.join(HERE, "ref_products_mixed_10x12x8.npz"), **rec)
    shutil.rmtree(base)


def svd_fixtures():
    base = tempfile.mkdtemp(prefix="plume_golden_")
    # snapshot path one character longer than the reduced path, so that the
    # reference's singular-value file name rule yields "<stream>.matrix"
    snap, red, scr = base + "/snap/", base + "/red/", base + "/scratch/"
    os.makedirs(snap)
    p = _abi.default_params(res=(10, 12, 8), vorticity_eps=1.0)
    subprocess.run(ref_args(p, 12, "column", snap) + ["streams=1"] +
                   moving_args((0.5, 0.35, 0.5), (0.4, 0.3, 0.35), 2.0, 3.0, True),
                   check=True, capture_output=True)
    cfg = base + "/svd.cfg"
    with open(cfg, "w") as f:
        f.write("snapshot path = %s\nreduced path = %s\nscratch path = %s\n"
                "simulation snapshots = 12\nreduced snapshots = 12\ndiscard threshold = 1e-9\n"
                "iop = 1\n" % (snap, red, scr))
    r = subprocess.run([SVD_REF, cfg], check=True, capture_output=True, text=True)
    out = {"threshold": 1e-9}
    for name, tag in zip(SVD_STREAMS, SVD_TAGS):
        pre = snap + name + ".matrix"
        out["dims_" + tag] = np.fromfile(pre + ".dims", dtype="<i4")
        out["stream_" + tag] = np.fromfile(pre + ".transpose")
        u = red + "U." + tag + ".matrix"
        hdr = np.fromfile(u, dtype="<i4", count=2)
        out["U_" + tag] = np.fromfile(u, dtype="<f8", offset=8).reshape(int(hdr[0]), int(hdr[1]))
        sv = scr + name + ".matrix.singularValues.vector"
        nsv = int(np.fromfile(sv, dtype="<i4", count=1)[0])
        out["pca_" + tag] = np.fromfile(sv, dtype="<f8", offset=4, count=nsv)
        out["pca_file_bytes_" + tag] = os.path.getsize(red + "pca." + tag + ".vector")
    diffs = [float(l.split(":")[1]) for l in r.stdout.splitlines() if l.strip().startswith("Diff")]
    out["verify_diffs"] = np.array(diffs)
    np.savez_compressed(os.path.join(HERE, "ref_svd_10x12x8.npz"), **out)
    shutil.rmtree(base)
    print("svd fixture:", {t: out["U_" + t].shape for t in SVD_TAGS})


def plume_fixtures():
    for name, (kw, steps, src) in CASES.items():
        p = _abi.default_params(**kw)
        d, iters, fields = run_ref(p, steps, src)
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), iters=np.array(iters),
                            steps=steps, **params_record(p), **fields)
        shutil.rmtree(d)
        print(name, "iters", iters)

    # format fixtures: the reference's own state file and streams
    fx = os.path.join(HERE, "ref_state_8x10x6")
    shutil.rmtree(fx, ignore_errors=True)
    os.makedirs(fx)
    p = _abi.default_params(res=(8, 10, 6), vorticity_eps=1.0)
    d = tempfile.mkdtemp(prefix="plume_golden_")
    subprocess.run(ref_args(p, 2, "column", d) + ["gz=1", "streams=1"], check=True,
                   capture_output=True)
    for f in sorted(os.listdir(d)):
        if f.startswith("fluid.0001") or f.endswith(".dims") or f.endswith(".transpose"):
            shutil.copy(os.path.join(d, f), fx)
    subprocess.run([REF, "readgz", d + "/fluid.0001.fluid3d.gz", d + "/x"], check=True,
                   capture_output=True)
    fields = {n: np.fromfile(d + "/x.%s.f64" % n) for n in _abi.FIELDS}
    np.savez_compressed(os.path.join(fx, "fields.npz"), **fields, **params_record(p))
    shutil.rmtree(d)
    print("format fixture:", sorted(os.listdir(fx)))


def cfg1_fixture(steps=100):
    """The benchmark plume at 48x64x48 (configuration 1: FP64, the reference's
    own 1e-10 stop test), all of its steps, summarised."""
    res = (48, 64, 48)
    p = _abi.plume_config(res, precision=_abi.PREC_FP64, criterion=_abi.CRIT_REFERENCE, tol=1e-10)
    d, iters, fields = run_ref(p, steps, "box")
    out = dict(iters=np.array(iters), steps=steps, **params_record(p))
    for n in _abi.FIELDS:
        a = fields[n]
        out["sum_" + n] = a.sum()
        out["l2_" + n] = np.sqrt((a * a).sum())
        out["sample_" + n] = a[::97].copy()
    np.savez_compressed(os.path.join(HERE, "ref_cfg1_sampled.npz"), **out)
    shutil.rmtree(d)
    print("cfg1 iters", iters)


def moving_fixtures():
    for name, (kw, steps, src, c, l, per, tper, initvel) in MOVING.items():
        p = _abi.default_params(**kw)
        d, iters, fields = run_ref(p, steps, src, moving_args(c, l, per, tper, initvel))
        np.savez_compressed(os.path.join(HERE, "ref_moving_%s.npz" % name), iters=np.array(iters),
                            steps=steps, box_center=np.array(c), box_lengths=np.array(l),
                            period=per, translation_period=tper, initvel=int(initvel),
                            **params_record(p), **fields)
        shutil.rmtree(d)
        print("moving", name, "iters", iters)

    # format fixtures of a moving-box run: state file with postIOP and the
    # obstacle matrix, and the streams with the IOP rows and matrices
    fx = os.path.join(HERE, "ref_moving_state_10x12x8")
    shutil.rmtree(fx, ignore_errors=True)
    os.makedirs(fx)
    p = _abi.default_params(res=(10, 12, 8), vorticity_eps=1.0)
    mv = ((0.5, 0.35, 0.5), (0.4, 0.3, 0.35), 2.0, 3.0, True)
    d = tempfile.mkdtemp(prefix="plume_golden_")
    subprocess.run(ref_args(p, 2, "column", d) + ["gz=1", "streams=1"] + moving_args(*mv),
                   check=True, capture_output=True)
    for f in sorted(os.listdir(d)):
        if f.startswith("fluid.0001") or f.endswith(".dims") or f.endswith(".transpose") or \
                f.endswith(".matrices"):
            shutil.copy(os.path.join(d, f), fx)
    np.savez_compressed(os.path.join(fx, "box.npz"), box_center=np.array(mv[0]),
                        box_lengths=np.array(mv[1]), period=mv[2], translation_period=mv[3],
                        initvel=int(mv[4]), **params_record(p))
    shutil.rmtree(d)
    print("moving format fixture:", sorted(os.listdir(fx)))



if __name__ == "__main__":
    main()
