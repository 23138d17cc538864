#!/usr/bin/env python3
"""Throughput of the full-rank plume step (the reference's `fluid3D` stage).

Workload: the 128x192x128 plume -- closed box, box source with +-0.05 seeded
noise, buoyancy 1, vorticity 2 -- with FP32 fields and FP64 CG scalars, MIC(0)
PCG to a relative residual of 1e-6.  A "step" is one FLUID_3D_MIC::step
(source, buoyancy, vorticity confinement, advection, damping, projection).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Two arms run on the same plume: plain MIC(0)-PCG from p = 0 (the reference's
solve) and the learned warm start (the committed U-Net's guess, Galerkin
scaled, then the same MIC-PCG to the same stop test).  The metric compares
them; `value`, `e2e` and the roofline describe the learned arm, `arms` gives
both.

Prints one JSON line.  `value` is steps/s from CUDA events on the library's
stream around the K timed steps (state resident in HBM); `e2e` is steps/s
through the public API with the source values copied from pinned host memory
and the velocity snapshot (FP64, reference layout) copied back every step.
N > 1 runs N independent replicas (one per GPU, launched by torchrun); the
path has no data exchange between plumes.
"""
import argparse
import json
import math
import os
import statistics
import struct
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s, PCG iters/step @128x192x128: learned/FP32 vs plain MIC-PCG, res 1e-6"
RES = (128, 192, 128)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for N replicas (gloo over 127.0.0.1)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


# DRAM bytes (read + write) of one sweep launch from an ncu capture of this
# workload (dram__bytes.sum.per_second x gpu__time_duration.sum of one forward
# and one backward launch), keyed by grid and field bytes.
SWEEP_DRAM_BYTES = {((128, 192, 128), 4): 28.57e6}


def bytes_per_step(nint, iters, S, P):
    """Algorithmic HBM bytes of one step: each pass reads its operands once and
    writes its results once; 1 byte of cell flags per stencil pass."""
    return nint * (51 * S + 3 * P + 6 + iters * (16 * S + 2 * P + 3))


def bytes_per_iteration(nint, S, P):
    return nint * (16 * S + 2 * P + 3)


# Algorithmic bytes per interior cell of each stage outside the solve (the
# canonical model: each pass reads its operands and writes its results once,
# stencil neighbours from cache, wall flags one byte): the same figures the
# fluid3D step log uses.
STAGE_BYTES = {"forces": lambda S: 4 * S, "vorticity": lambda S: 18 * S + 2, "advection": lambda S: 10 * S,
               "damping": lambda S: 6 * S, "divergence": lambda S: 5 * S + 1, "gradient": lambda S: 7 * S}


def stage_roofline(stages, nint, S, peak):
    """Achieved GB/s and fraction of the measured HBM rate of each stencil
    stage from its mean device time."""
    out = {}
    for k, f in STAGE_BYTES.items():
        ms = stages.get(k, 0.0)
        gbs = f(S) * nint / (ms * 1e6) if ms > 0 else None
        out[k] = {"ms": ms, "achieved_gbs": gbs, "frac": (gbs / peak) if gbs else None,
                  "bytes_per_cell": f(S)}
    return out


def host_cpu():
    """(logical cores, model name) of this host."""
    model = None
    try:
        for line in open("/proc/cpuinfo"):
            k = line.split(":")[0].strip().lower()
            if k in ("model name", "cpu part") and model is None:
                model = line.split(":", 1)[1].strip()
    except OSError:
        pass
    return os.cpu_count(), model


def cpu_baseline(res, steps, skip=0):
    """The oracle (FP64 CPU restatement of the reference step, 1 thread, as
    the reference runs) on steps skip .. skip+steps-1 of the same plume, the
    first `skip` run untimed (the GPU arms' warm-up window): steps/s."""
    from cfs_plume_gb300 import _abi
    from oracle import oracle
    p = _abi.plume_config(res, precision=_abi.PREC_FP64)
    o = oracle.Oracle(p)
    for s in range(skip):
        o.add_source(s)
        o.step()
    t0 = time.perf_counter()
    iters = []
    for s in range(skip, skip + steps):
        o.add_source(s)
        iters.append(o.step().iterations)
    dt = time.perf_counter() - t0
    return steps / dt, iters, dt


def run_reference(args, rank, world):
    """--impl reference: the reference step's CPU implementation, timed on the
    host.  The reference sources are not present on the GPU host, so the
    oracle port (a line-by-line restatement pinned bit-for-bit to the
    reference) stands in; the reference step is single-threaded."""
    if rank != 0:
        return 0
    res = RES
    sample = max(1, min(args.steps, 3))
    skip = max(0, min(args.warmup, 5))
    v, iters, dt = cpu_baseline(res, sample, skip)
    cores, model = host_cpu()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": world,
        "steps": sample, "warmup": skip, "ms_per_step": 1000.0 / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "plume 128x192x128, closed box, box source +-0.05 seeded noise, "
                               "buoyancy 1, vorticity 2, MIC(0)-PCG rel-residual 1e-6",
                   "res": list(res)},
        "pcg_iters_per_step": statistics.mean(iters),
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                         "host_cores": cores, "host_cpu": model,
                         "sample": "steps %d-%d of the same plume after %d untimed warm-up steps, as the GPU "
                                   "arms' timed window starts (%.1f s, %s PCG iterations); the reference step "
                                   "is single-threaded" % (skip, skip + sample - 1, skip, dt, iters)},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_arm(g, a, dist, nbox, box_values_seed):
    """Warm-up, then K device-timed steps (CUDA events on the library stream,
    MIC sweep launches bracketed by events), then the end-to-end loop through
    the public API with host buffers.  Returns a dict of raw measurements."""
    import numpy as np
    from cfs_plume_gb300 import _abi
    g.run_timed(0, a.warmup)
    dist.barrier()
    g.lib.plume_sync(g.h)
    # the timed steps: CG loop as one CUDA graph launch per solve
    ms, stats = g.run_timed(a.warmup, a.steps)
    dist.barrier()
    ms_max = dist.max(ms)
    # a second pass of K steps with CUDA events around every MIC sweep launch
    # (event records cannot sit inside the graph's loop body, so this pass
    # drives the CG loop from the host) for the sweep kernel's roofline
    g.profile_sweeps(True)
    g.run_timed(a.warmup + a.steps, a.steps)
    sweep_ms, sweep_launches = g.sweep_times()
    g.profile_sweeps(False)
    dist.barrier()
    n_e2e = a.e2e_steps if a.e2e_steps is not None else max(3, min(a.steps, 10))
    rng = np.random.default_rng(box_values_seed)
    src = [1.0 + 0.05 * (2.0 * rng.random(nbox) - 1.0) for _ in range(n_e2e)]
    vel = np.empty(3 * g.N)
    dist.barrier()
    t0 = time.perf_counter()
    for k in range(n_e2e):
        g.add_source_values(src[k])
        g.step(stats=False)
        g.lib.plume_download(g.h, _abi.FIELD_ID["velocity"], vel.ctypes.data, vel.size)
    e2e_s = dist.max(time.perf_counter() - t0)
    dist.barrier()
    iters = [s.iterations for s in stats]
    stages = {k: statistics.mean(getattr(s, "ms_" + k) for s in stats) for k in _abi.STAGES}
    return {"ms": ms_max, "value": dist.sum(a.steps) / (ms_max / 1000.0), "iters": iters, "stages": stages,
            "launches": sum(s.launches for s in stats), "ms_solve": sum(s.ms_solve for s in stats),
            "fallbacks": sum(s.fallback for s in stats),
            "max_rel_residual": max(s.rel_residual for s in stats),
            "sweep_ms": sweep_ms, "sweep_launches": sweep_launches,
            "e2e": dist.sum(n_e2e) / e2e_s, "n_e2e": n_e2e}


# the moving box of the stepWithMovingObstacle measurement (cellCenter units)
MOVING_BOX = dict(center=(0.5, 0.3, 0.5), lengths=(0.35, 0.1, 0.2), period=2.0, translation_period=4.0)


def measure_moving(a, dist, res, prec, local, rank):
    """stepWithMovingObstacle on the same plume with a spinning, swaying box:
    K device-timed steps (CG loop as a CUDA graph), then K more with CUDA
    events around every stomp launch for the stomp kernel's roofline."""
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import BOX, Plume
    g = Plume(_abi.plume_config(res, precision=prec, seed=rank, device=local))
    mb = MOVING_BOX
    box = BOX(mb["center"], mb["lengths"], mb["period"], mb["translation_period"])
    box.set_dt(0.1)
    g.run_moving_timed(box, 0, a.warmup, stats=False)
    dist.barrier()
    g.lib.plume_sync(g.h)
    ms, stats = g.run_moving_timed(box, a.warmup, a.steps)
    dist.barrier()
    ms_max = dist.max(ms)
    g.profile_sweeps(True)
    g.run_moving_timed(box, a.warmup + a.steps, a.steps, stats=False)
    stomp_ms, stomp_n = g.stomp_times()
    g.profile_sweeps(False)
    inside = int(g.iop()[0].sum())
    g.close()
    return {"ms": ms_max, "value": dist.sum(a.steps) / (ms_max / 1000.0),
            "iters": [s.iterations for s in stats], "launches": sum(s.launches for s in stats),
            "converged": all(s.converged for s in stats), "stomp_ms": stomp_ms,
            "stomp_launches": stomp_n, "inside": inside}


def measure_snapshot_svd(res, prec, local, rank, snaps):
    """svdOutOfCoreMultiple on the device: `snaps` steps of the same plume with
    the velocity.final row kept in HBM after each (plume_snapshots), then the
    in-place QR, SVD of R and U = Q U_R (timed by CUDA events inside)."""
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, Snapshots
    g = Plume(_abi.plume_config(res, precision=prec, seed=rank, device=local))
    sn = Snapshots(g, "final", snaps)
    for s in range(snaps):
        g.add_source(s)
        g.step(stats=False)
        sn.append()
    rows, cols = sn.dims()
    t0 = time.perf_counter()
    pca, kept, info = sn.svd(1e-9, u_path=None)
    wall = time.perf_counter() - t0
    sn.close()
    g.close()
    return {"rows": rows, "cols": cols, "kept": kept, "info": info, "wall_s": wall}


def hyperplanes(res):
    """i + j + k hyperplanes of the interior: the length of the MIC(0)
    recurrence's dependency chain (440 at 128x192x128)."""
    return sum(int(v) - 2 for v in res) - 2


def _write_eigen(path, M):
    """EIGEN::write layout: int32 rows, cols, then the row-major doubles."""
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", M.shape[0], M.shape[1]))
        M.astype("<f8").tofile(f)


def measure_reduced(steps, local, rank, res=(64, 96, 64), rank_r=32, points=2000):
    """buildOutOfCoreMatrices and stepReorderedCubatureStam on the GPU with a
    synthetic reduced model of the reference's file layout (seeded random
    bases of rank 32, the projected operators built from them on the device,
    2000 seeded cubature cells), FP32 plume fields."""
    import numpy as np
    import shutil
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, ReducedModel, build_products
    nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
    n = 3 * nint
    rng = np.random.default_rng(7 + rank)
    d = tempfile.mkdtemp(prefix="plume_reduced_bench_")
    try:
        for fn in ("U.preadvect.matrix", "U.final.matrix", "U.prediffuse.matrix", "U.preproject.matrix"):
            _write_eigen(os.path.join(d, fn), rng.standard_normal((n, rank_r)) / math.sqrt(n))
        _write_eigen(os.path.join(d, "U.pressure.matrix"), rng.standard_normal((nint, rank_r)) / math.sqrt(nint))
        cells = np.sort(rng.choice(nint, points, replace=False)).astype("<i4")
        with open(os.path.join(d, "cubature"), "wb") as f:
            f.write(struct.pack("<i", points))
            cells.tofile(f)
            np.full(points, nint / points, dtype="<f8").tofile(f)
        g = Plume(_abi.plume_config(res, precision=_abi.PREC_FP32, seed=rank, device=local))
        build_products(g, d)  # warm-up (module load, first allocations)
        products = build_products(g, d)
        m = ReducedModel(g, d)
        for s in range(3):
            g.add_source(s)
            m.step()
        tot = red = 0.0
        launches = 0
        for s in range(steps):
            g.add_source(3 + s)
            st = m.step()
            tot += st.ms_total
            red += st.ms_solve
            launches += st.launches
        m.close()
        g.close()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"res": res, "n": n, "r": rank_r, "points": points, "ms_total": tot / steps, "ms_reduced": red / steps,
            "launches": launches / steps, "products": products}


def products_record(r, fp64_peak_tflops):
    """The projected-operator build of the same synthetic model."""
    p = r["products"]
    ach = p["gflop"] / p["ms_device"] if p["ms_device"] > 0 else None  # GFLOP/ms = TFLOP/s
    return {"workload": "buildOutOfCoreMatrices, plume %dx%dx%d walls, four synthetic rank-%d FP64 bases "
                        "(U.pressure, U.preproject, U.prediffuse, U.final)" % (tuple(r["res"]) + (r["r"],)),
            "ms_device": p["ms_device"], "ms_total_with_file_io": p["ms_total"], "gflop": p["gflop"],
            "roofline": {"bound": "fp64", "kernel": "whole build (stencils, k_atb projections, Gauss-Jordan)",
                         "achieved": ach, "peak": fp64_peak_tflops, "unit": "TFLOP/s",
                         "frac": (ach / fp64_peak_tflops) if ach else None,
                         "flops_model": "sum of 2 K a b over the projections + 4 r^3 for the inverse"}}


def reduced_record(r, peak):
    # the reduced part reads U_pa and U_f once each (n x r doubles), the
    # peeled velocity (3 N_int floats) and writes it back
    bytes_red = 2 * r["n"] * r["r"] * 8 + 2 * r["n"] * 4
    ach = bytes_red / (r["ms_reduced"] / 1000.0) / 1e9 if r["ms_reduced"] > 0 else None
    return {"workload": "stepReorderedCubatureStam, plume %dx%dx%d FP32 fields, synthetic reduced model: rank %d "
                        "bases (FP64), %d cubature points" % (tuple(r["res"]) + (r["r"], r["points"])),
            "value": 1000.0 / r["ms_total"], "unit": "steps/s", "ms_per_step": r["ms_total"],
            "ms_reduced_part": r["ms_reduced"], "launches_per_step": r["launches"],
            "roofline": {"bound": "hbm", "kernel": "reduced part (projection, cubature, unprojection)",
                         "achieved": ach, "peak": peak, "unit": "GB/s", "frac": (ach / peak) if ach else None,
                         "bytes_model": "2 n r 8 + 2 n 4 per step (n = 3 N_int)"}}


def svd_record(r, fp64_peak_tflops):
    n, m = r["cols"], r["rows"]
    info = r["info"]
    qr_flops = 2.0 * n * m * m          # MGS: a dot and an axpy per column pair
    qr_bytes = 8.0 * n * m * m          # each pass reads and writes the later columns
    qr_s = info["ms_qr"] / 1000.0
    ach = qr_flops / qr_s / 1e12 if qr_s > 0 else None
    return {"workload": "velocity.final snapshots of the same plume kept in HBM (n = 3 N_int = %d, m = %d), "
                        "Gram-Schmidt QR + one-sided Jacobi SVD of R in FP64, U not formed" % (n, m),
            "kept": r["kept"], "ms_qr": info["ms_qr"], "ms_svd_of_r": info["ms_svd"],
            "jacobi_sweeps": info["sweeps"], "wall_s": r["wall_s"],
            "roofline": {"bound": "fp64", "kernel": "k_mgs_pass (Gram-Schmidt pass)",
                         "achieved": ach, "peak": fp64_peak_tflops, "unit": "TFLOP/s",
                         "frac": (ach / fp64_peak_tflops) if ach else None,
                         "peak_kind": "derived: 2 FP64 FMA/clock/SM (ncu dfma peak_sustained) x 152 SMs x 2070 MHz",
                         "flops_model": "2 n m^2", "bytes_model": "8 n m^2",
                         "achieved_gbs": qr_bytes / qr_s / 1e9 if qr_s > 0 else None}}


def measure_batched(steps, warmup, seed=0, n=64):
    """The batched-plume configuration: `n` randomised plumes of uneven grids
    (plume_batch_params: 32^3 .. 96x128x96, source position, buoyancy and
    vorticity drawn per instance), FP32 fields, MIC(0)-PCG rel-L2 1e-6,
    stepped together (plume_batch_run).  Aggregate interior cell-steps/s of
    the fused engine (one launch per stage over all plumes, each step one
    CUDA graph launch, tile shapes from the autotuner), with the streams
    engine (one handle and stream per plume) on the same plumes beside it."""
    import numpy as np
    from cfs_plume_gb300.batch import PlumeBatch, batch_params
    params = [batch_params(seed, i) for i in range(n)]
    cells = np.array([(p.res[0] - 2) * (p.res[1] - 2) * (p.res[2] - 2) for p in params], dtype=np.float64)
    arms = {}
    for engine in ("fused", "fused_one_group", "streams"):
        t0 = time.time()
        if engine == "fused_one_group":  # the same lockstep CG without the group overlap
            b = PlumeBatch(params, engine="fused", groups=1)
        else:
            b = PlumeBatch(params, engine=engine)
        create_s = time.time() - t0
        b.run(0, warmup, stats=False)
        secs, stats = b.run(warmup, steps, stats=True)
        tuning = b.tuning() if engine != "streams" else None
        b.close()
        # the canonical bytes model per plume and step (FP32 fields, each plume's own iterations)
        model_bytes = sum(bytes_per_step(cells[i], st.iterations, 4, 4) for i in range(n) for st in stats[i])
        arm = {"value": cells.sum() * steps / secs, "seconds": secs, "create_seconds": create_s,
               "instance_steps_per_s": n * steps / secs,
               "achieved_gbs": model_bytes / secs / 1e9,
               "pcg_iters_per_step_mean": float(np.mean([[s.iterations for s in st] for st in stats])),
               "pcg_iters_per_step_max": int(np.max([[s.iterations for s in st] for st in stats])),
               "all_converged": all(s.converged for st in stats for s in st)}
        if engine != "streams":
            # one graph launch per step; the statistics row carries the
            # kernels its step launched and the device time of the call
            arm["gpu_launches_per_step"] = float(np.mean([s.launches for s in stats[0]]))
            arm["device_seconds"] = sum(s.ms_total for s in stats[0]) / 1e3
            arm["tuning"] = tuning
        arms[engine] = arm
    grids = {}
    for p in params:
        k = "x".join(str(v) for v in p.res)
        grids[k] = grids.get(k, 0) + 1
    f = arms["fused"]
    peak, peak_kind = measured_peaks()
    return {"value": f["value"], "unit": "interior cell-steps/s", "engine": "fused", "instances": n,
            "steps": steps, "warmup": warmup, "seconds": f["seconds"],
            "achieved_gbs": f["achieved_gbs"], "hbm_frac": f["achieved_gbs"] / peak, "peak_gbs": peak,
            "bytes_model": "per plume and step N_int*(51S+3P+6 + iters*(16S+2P+3)), S = P = 4",
            "instance_steps_per_s": f["instance_steps_per_s"],
            "pcg_iters_per_step_mean": f["pcg_iters_per_step_mean"], "all_converged": f["all_converged"],
            "fused_over_streams": f["value"] / arms["streams"]["value"], "arms": arms, "grids": grids,
            "interior_cells_total": float(cells.sum()),
            "workload": "%d randomised closed-box plumes of the batched configuration, FP32 fields, "
                        "MIC(0)-PCG rel-L2 1e-6, advanced in lockstep: one launch per stage over all "
                        "plumes, each step one CUDA graph launch" % n}


def measure_with_output(local, rank, cfg1_steps=20, big_steps=2):
    """The step with its output on: the state file (writeGz layout, gzip level
    1, deflated in parallel on the host) and the six stream rows written each
    step by the handle's asynchronous writer, as fluid3D writes them
    (fluid3D.cpp:357-398).  Two workloads: config 1 (48x64x48 FP64, rel-L2
    1e-10, output every step) and the 128x192x128 FP32 plume.  Wall-clock
    steps/s with and without the output, the bytes written per step; the files
    go to a temporary directory that is removed afterwards."""
    import shutil
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    out = {}
    for name, res, prec, tol, steps in (
            ("config1_48x64x48_fp64", (48, 64, 48), _abi.PREC_FP64, 1e-10, cfg1_steps),
            ("plume_128x192x128_fp32", RES, _abi.PREC_FP32, 1e-6, big_steps)):
        rec = {}
        for with_out in (False, True):
            d = tempfile.mkdtemp(prefix="plume_out_")
            g = None
            try:
                g = Plume(_abi.plume_config(res, precision=prec, tol=tol, seed=rank, device=local))
                warm = 2
                for s in range(warm):
                    g.add_source(s)
                    g.step()
                    if with_out:
                        g.snapshot_async(d, s)
                if with_out:
                    g.wait_snapshots()
                g.sync()
                before = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
                t0 = time.time()
                for s in range(warm, warm + steps):
                    g.add_source(s)
                    g.step()
                    if with_out:
                        g.snapshot_async(d, s)
                if with_out:
                    g.wait_snapshots()
                g.sync()
                secs = time.time() - t0
                written = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d)) - before
                key = "with_output" if with_out else "no_output"
                rec[key] = {"steps_per_s": steps / secs, "steps": steps}
                if with_out:
                    rec[key]["bytes_written_per_step"] = written / steps
            except Exception as e:  # a full disk on the host must not end the bench line
                rec["with_output" if with_out else "no_output"] = {"error": str(e)[:200]}
            finally:
                if g is not None:
                    g.close()
                shutil.rmtree(d, ignore_errors=True)
        rec["workload"] = ("%dx%dx%d %s, rel-L2 %.0e, closed box, box source; the state file and the "
                           "stream rows each step through plume_snapshot_async, wall clock incl. the "
                           "last write" % (res + ("FP64" if prec == _abi.PREC_FP64 else "FP32", tol)))
        out[name] = rec
    return out


LARGE_RES = (256, 384, 256)


def measure_large(steps, warmup, weights, local, rank):
    """The large plume of the same family (256x384x256, ~25M cells, the
    source box scaled the same way), FP32 fields, rel-L2 1e-6: plain MIC-PCG
    and the learned warm start with the network trained on 64x96x64 plumes
    (no retraining), `steps` device-timed steps after `warmup`."""
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    out = {}
    for arm in ("plain", "learned"):
        if arm == "learned" and not os.path.exists(weights):
            continue
        g = Plume(_abi.plume_config(LARGE_RES, seed=rank, device=local,
                                    warm_start=_abi.WARM_LEARNED if arm == "learned" else _abi.WARM_ZERO))
        net = None
        if arm == "learned":
            from cfs_plume_gb300.net import PlumeNet
            net = PlumeNet(device=local, path=weights)
            net.attach(g)
        g.run_timed(0, warmup, stats=False)
        ms, stats = g.run_timed(warmup, steps)
        g.close()
        if net is not None:
            net.close()
        out[arm] = {"value": 1000.0 * steps / ms, "unit": "steps/s", "ms_per_step": ms / steps,
                    "pcg_iters_per_step": statistics.mean(s.iterations for s in stats),
                    "fallbacks": sum(s.fallback for s in stats),
                    "all_converged": all(s.converged for s in stats)}
    rec = {"workload": "plume %dx%dx%d (~25M cells), closed box, box source +-0.05 seeded noise, buoyancy 1, "
                       "vorticity 2, FP32 fields, MIC(0)-PCG rel-residual 1e-6; learned: the warm-start network "
                       "trained on 64x96x64 plumes, not retrained" % LARGE_RES,
           "steps": steps, "warmup": warmup, "arms": out}
    if "learned" in out:
        rec["learned_over_plain"] = out["learned"]["value"] / out["plain"]["value"]
    return rec


def net_forward_mode(spec, warmup=3, iters=5):
    """--net-forward X,Y,Z: wall time of the warm-start network's forward pass
    (host input in, host output out) on a seeded standard-normal field with
    the committed weights: `warmup` untimed passes, then `iters` timed ones.
    PLUME_CONV_TC=0 runs every convolution on the mma.sync kernel."""
    import numpy as np
    from cfs_plume_gb300.net import PlumeNet
    res = tuple(int(v) for v in spec.split(","))
    net = PlumeNet(seed=0, path=os.path.join(ROOT, "cfs_plume_gb300", "weights", "unet_warmstart.bin"))
    x = np.random.default_rng(0).standard_normal((1, res[2], res[1], res[0])).astype(np.float32)
    for _ in range(warmup):
        net.forward(x, res)
    t0 = time.perf_counter()
    for _ in range(iters):
        y = net.forward(x, res)
    ms = (time.perf_counter() - t0) / max(1, iters) * 1000.0
    net.close()
    print(json.dumps({"res": res, "forward_ms_wall": ms, "mean_abs_output": float(np.abs(y).mean()),
                      "tcgen05": os.environ.get("PLUME_CONV_TC", "1") != "0"}), flush=True)
    return 0


SWEEP_SCALING_RES = [(130, 194, 18), (130, 194, 34), (130, 194, 66), (130, 194, 130), (130, 98, 130),
                     (130, 50, 130), (130, 386, 66)]


def sweep_scaling_mode(iters=20):
    """--sweep-scaling: device time per MIC(0) sweep launch (CUDA events from
    plume_profile_sweeps around plume_mic_apply) on FP32 handles whose
    interior is 128 cells wide (4 cells per lane), varying the rows per plane
    (interior ny + 31) and the plane count (interior nz), then the least-squares
    fit t = a + b R + c nz: b is the cost of one row step of a warp, c the lag
    the wavefront adds per plane."""
    import numpy as np
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    rows = []
    for res in SWEEP_SCALING_RES:
        g = Plume(_abi.default_params(res=res, bc=(1, 1, 1, 1, 1, 1), precision=_abi.PREC_FP32))
        r = np.random.default_rng(0).standard_normal(g.N)
        g.mic_apply(r)
        g.profile_sweeps(True)
        for _ in range(iters):
            g.mic_apply(r)
        ms, n = g.sweep_times()
        g.profile_sweeps(False)
        g.close()
        rows.append({"res": res, "rows": res[1] - 2 + 31, "planes": res[2] - 2, "us_per_sweep": ms / n * 1e3})
    A = np.array([[1.0, q["rows"], q["planes"]] for q in rows])
    y = np.array([q["us_per_sweep"] for q in rows])
    coef = np.linalg.lstsq(A, y, rcond=None)[0]
    print(json.dumps({"sweeps": rows, "fit_us": {"const": coef[0], "per_row": coef[1], "per_plane": coef[2]},
                      "fit_max_abs_residual_us": float(np.abs(A @ coef - y).max())}), flush=True)
    return 0


def products_mode(spec, rank=32, warmup=1, iters=1):
    """--products X,Y,Z: the projected-operator build of a reduced model
    (buildOutOfCoreMatrices, plume_reduced_build_products) on seeded
    synthetic bases of `rank` columns (U.pressure N_int rows, U.preproject,
    U.prediffuse, U.final 3 N_int), reference default walls."""
    import numpy as np
    import shutil
    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume, build_products
    res = tuple(int(v) for v in spec.split(","))
    nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
    rng = np.random.default_rng(11)
    d = tempfile.mkdtemp(prefix="plume_products_") + "/"
    try:
        _write_eigen(d + "U.pressure.matrix", rng.standard_normal((nint, rank)) / math.sqrt(nint))
        for fn in ("U.preproject.matrix", "U.prediffuse.matrix", "U.final.matrix"):
            _write_eigen(d + fn, rng.standard_normal((3 * nint, rank)) / math.sqrt(3 * nint))
        g = Plume(_abi.default_params(res=res))
        for _ in range(warmup):
            build_products(g, d)
        dev = wall = 0.0
        info = None
        for _ in range(iters):
            info = build_products(g, d)
            dev += info["ms_device"]
            wall += info["ms_total"]
        g.close()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    n = max(1, iters)
    print(json.dumps({"res": res, "rank": rank, "ms_device": dev / n, "ms_total": wall / n,
                      "gflop": info["gflop"], "tflops": info["gflop"] / (dev / n) if dev > 0 else None}),
          flush=True)
    return 0


def moving_record(m, res, N, nint, S, peak, steps):
    # the stomp reads every velocity (border cells for the postIOP copy), writes
    # postIOP everywhere, the inside mask on the interior, and inside the box
    # the new velocity and the obstacle matrix's last column (FP64)
    stomp_bytes = N * 6 * S + nint + m["inside"] * (3 * S + 24)
    avg = m["stomp_ms"] / m["stomp_launches"] if m["stomp_launches"] else None
    ach = stomp_bytes / (avg / 1000.0) / 1e9 if avg else None
    mb = MOVING_BOX
    return {"value": m["value"], "unit": "steps/s", "ms_per_step": m["ms"] / steps,
            "pcg_iters_per_step": statistics.mean(m["iters"]), "all_converged": m["converged"],
            "workload": "stepWithMovingObstacle on the plume %dx%dx%d (no buoyancy), plain MIC(0)-PCG "
                        "from p = 0, box centre %s lengths %s spin period %g sway period %g, "
                        "spun and translated after every step" % (res + (mb["center"], mb["lengths"],
                                                                         mb["period"],
                                                                         mb["translation_period"])),
            "inside_cells": m["inside"],
            "roofline": {"bound": "hbm", "kernel": "k_box_stomp (obstacle stomp, postIOP copy)",
                         "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": (ach / peak) if ach else None, "bytes_per_launch": stomp_bytes,
                         "ms_per_launch": avg, "launches_timed": m["stomp_launches"],
                         "bytes_model": "N*6S + N_int + inside*(3S+24)"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", default=None, help="X,Y,Z (default 128,192,128)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--cpu-steps", type=int, default=3, help="oracle steps for cpu_baseline (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--arms", default="both", choices=["both", "plain"],
                    help="both: plain MIC-PCG and the learned warm start (the headline value)")
    ap.add_argument("--weights", default=None, help="warm-start network (default: the committed one)")
    ap.add_argument("--no-moving", action="store_true", help="skip the moving-box step measurement")
    ap.add_argument("--no-learned-pc", action="store_true",
                    help="skip the arm with the network as the flexible-CG preconditioner")
    ap.add_argument("--svd-snapshots", type=int, default=48,
                    help="snapshots for the device snapshot-SVD measurement (0: skip)")
    ap.add_argument("--no-reduced", action="store_true", help="skip the reduced-step measurement")
    ap.add_argument("--large-steps", type=int, default=5,
                    help="timed steps of the 256x384x256 plume, plain and learned (0: skip)")
    ap.add_argument("--no-output", action="store_true",
                    help="skip the measurement of the step with its state file and streams written")
    ap.add_argument("--batch-steps", type=int, default=10,
                    help="timed steps of the 64-plume batched configuration (0: skip)")
    ap.add_argument("--net-forward", default=None, metavar="X,Y,Z",
                    help="only time the network's forward pass at this grid")
    ap.add_argument("--products", default=None, metavar="X,Y,Z",
                    help="only time the projected-operator build at this grid")
    ap.add_argument("--sweep-scaling", action="store_true",
                    help="only time the MIC sweep against rows and planes per plume (and fit)")
    a = ap.parse_args()
    rank, world, local = dist_env()
    if a.impl == "reference":
        return run_reference(a, rank, world)
    if a.net_forward:
        return net_forward_mode(a.net_forward)
    if a.products:
        return products_mode(a.products)
    if a.sweep_scaling:
        return sweep_scaling_mode()
    a.warmup = max(a.warmup, 3)

    from cfs_plume_gb300 import _abi
    from cfs_plume_gb300.plume import Plume
    import numpy as np

    res = tuple(int(v) for v in a.res.split(",")) if a.res else RES
    prec = _abi.PREC_FP32 if a.precision == "fp32" else _abi.PREC_FP64
    S = 4 if prec == _abi.PREC_FP32 else 8
    P = S
    dist = Dist(world)
    p = _abi.plume_config(res, precision=prec, seed=rank, device=local)
    nint = (res[0] - 2) * (res[1] - 2) * (res[2] - 2)
    lo, hi = p.box_lo, p.box_hi
    nbox = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2])
    weights = a.weights if a.weights else os.path.join(ROOT, "cfs_plume_gb300", "weights", "unet_warmstart.bin")
    learned = os.path.exists(weights) and a.arms != "plain"

    # both arms on the same plume (same seed and source values); clocks are
    # sampled from the first timed step to the last
    clocks = ClockSampler(local)
    clocks.start()
    g = Plume(p)
    plain = measure_arm(g, a, dist, nbox, rank)
    g.close()
    prev = None
    if a.arms != "plain":  # the previous step's pressure as the guess, no network
        gp = Plume(_abi.plume_config(res, precision=prec, seed=rank, device=local,
                                     warm_start=_abi.WARM_PREVIOUS))
        prev = measure_arm(gp, a, dist, nbox, rank)
        gp.close()
    lrn = lpc = None
    if learned:
        from cfs_plume_gb300.net import PlumeNet
        net = PlumeNet(device=local, path=weights)
        gl = Plume(_abi.plume_config(res, precision=prec, seed=rank, device=local,
                                     warm_start=_abi.WARM_LEARNED))
        net.attach(gl)
        lrn = measure_arm(gl, a, dist, nbox, rank)
        gl.close()
        if not a.no_learned_pc:
            # the network as the preconditioner stage: flexible CG with
            # z = net(r), started from the previous pressure
            gpc = Plume(_abi.plume_config(res, precision=prec, seed=rank, device=local,
                                          warm_start=_abi.WARM_PREVIOUS, preconditioner=_abi.PRECOND_NET))
            net.attach(gpc)
            lpc = measure_arm(gpc, a, dist, nbox, rank)
            gpc.close()
        net.close()
    mov = None if a.no_moving else measure_moving(a, dist, res, prec, local, rank)
    svd = measure_snapshot_svd(res, prec, local, rank, a.svd_snapshots) if a.svd_snapshots > 0 else None
    red = None if a.no_reduced else measure_reduced(a.steps, local, rank)
    bat = measure_batched(a.batch_steps, 3, seed=rank) if a.batch_steps > 0 else None
    big = measure_large(a.large_steps, 3, weights, local, rank) if a.large_steps > 0 else None
    wout = None if a.no_output else measure_with_output(local, rank)
    clk = clocks.stop()
    head = lrn if lrn is not None else plain
    ms_max, value, iters = head["ms"], head["value"], head["iters"]
    launches, ms_solve = head["launches"], head["ms_solve"]
    sweep_ms, sweep_launches = head["sweep_ms"], head["sweep_launches"]
    e2e = head["e2e"]
    N = res[0] * res[1] * res[2]

    peak, peak_kind = measured_peaks()
    mean_iters = statistics.mean(iters)
    step_bytes = bytes_per_step(nint, mean_iters, S, P)
    solve_bytes = sum(nint * (5 * S + 2 * P + 2) + it * bytes_per_iteration(nint, S, P) for it in iters)
    achieved_solve = solve_bytes / (ms_solve / 1000.0) / 1e9 if ms_solve > 0 else None
    # dominant kernel: one MIC sweep launch reads r (or q) and the diagonal and
    # writes q (or z) once per interior cell
    sweep_bytes = nint * (2 * S + P)
    sweep_avg_ms = sweep_ms / sweep_launches if sweep_launches else None
    achieved_sweep = sweep_bytes / (sweep_avg_ms / 1000.0) / 1e9 if sweep_avg_ms else None
    traffic = SWEEP_DRAM_BYTES.get((res, S))

    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if S == 4 else "f64",
        "data": "synthetic",
        "config": {"workload": "plume %dx%dx%d, closed box, box source +-0.05 seeded noise, "
                               "buoyancy 1, vorticity 2, MIC(0)-PCG rel-residual 1e-6" % res,
                   "res": list(res),
                   "solver": ("MIC(0)-PCG from the learned warm start: A-norm Galerkin combination of "
                              "the U-Net guess and the previous pressure (plain fallback)" if lrn
                              else "plain MIC(0)-PCG from p = 0"),
                   "precision": "FP32 fields, FP64 CG scalars/MIC diagonal" if S == 4 else "FP64",
                   "l2": "step working set %.0f MB > 129 MB L2 (no flush needed)" %
                         (37 * S * N / 1e6),
                   "parallelism": "replicas" if world > 1 else "single"},
        "pcg_iters_per_step": mean_iters,
        # the metric's comparison: learned solver over plain MIC-PCG at the
        # same stop test, steps/s and PCG iterations per step
        "learned_over_plain": (lrn["value"] / plain["value"]) if lrn else None,
        "learned_iters_over_plain": (statistics.mean(lrn["iters"]) / statistics.mean(plain["iters"]))
                                    if lrn else None,
        "target_learned_over_plain": 3.0,
        "learned_pc_over_plain": (lpc["value"] / plain["value"]) if lpc else None,
        "arms": {name: {"value": r["value"], "unit": "steps/s", "ms_per_step": r["ms"] / a.steps,
                        "pcg_iters_per_step": statistics.mean(r["iters"]), "fallbacks": r["fallbacks"],
                        "max_rel_residual": r["max_rel_residual"], "e2e": r["e2e"],
                        "ms_stages": r["stages"]}
                 for name, r in (("plain", plain), ("previous", prev), ("learned", lrn), ("learned_pc", lpc))
                 if r is not None},
        "achieved_gbs_step": step_bytes / (ms_max / a.steps / 1000.0) / 1e9,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_mic_wave_cl (MIC(0) forward/backward sweep)",
                     "achieved": achieved_sweep, "peak": peak, "unit": "GB/s",
                     "frac": (achieved_sweep / peak) if achieved_sweep else None,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "bytes_per_launch": sweep_bytes, "ms_per_launch": sweep_avg_ms,
                     "launches_timed": sweep_launches,
                     "bytes_model": "N_int*(2S+P) per sweep launch",
                     "note": "latency-bound dependency chain (i+j+k wavefront); HBM roof for reference",
                     # the recurrence's i+j+k hyperplanes over the interior, and
                     # the sweep time per hyperplane stage
                     "hyperplanes_per_sweep": hyperplanes(res),
                     "ns_per_hyperplane": (sweep_avg_ms * 1e6 / hyperplanes(res)) if sweep_avg_ms else None,
                     "pass": "second pass of K steps with CUDA events around each sweep launch "
                             "(host-driven CG loop); value is timed with the CG loop as a CUDA graph"},
        "stage_roofline": dict(stage_roofline(head["stages"], nint, S, peak),
                               note="per stencil stage of the headline arm: mean CUDA-event time, algorithmic "
                                    "bytes per interior cell x N_int; neighbour stencils as shared-memory "
                                    "halo tiles, forces and advection grid-stride; HBM-bound"),
        "solve_roofline": {"kernel": "poisson solve (all MIC-PCG kernels)", "achieved": achieved_solve,
                           "unit": "GB/s", "frac": (achieved_solve / peak) if achieved_solve else None,
                           "bytes_model": "N_int*(5S+2P+2 + iters*(16S+2P+3)) per solve"},
        "moving_box": moving_record(mov, res, N, nint, S, peak, a.steps) if mov else None,
        "snapshot_svd": svd_record(svd, 2 * 2 * 152 * 2.070e9 / 1e12) if svd else None,
        "reduced_step": reduced_record(red, peak) if red else None,
        "reduced_products": products_record(red, 2 * 2 * 152 * 2.070e9 / 1e12) if red else None,
        "batched": bat,
        "large_plume": big,
        "with_output": wout,
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": nbox * 8,
                "d2h_bytes_per_step": 3 * N * 8},
        "clocks": clk,
    }
    if rank == 0 and a.cpu_steps > 0:
        skip = min(a.warmup, 5)
        v, it_cpu, dt = cpu_baseline(res, a.cpu_steps, skip)
        cores, model = host_cpu()
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                                "host_cores": cores, "host_cpu": model,
                                "sample": "steps %d-%d of the same plume after %d untimed warm-up steps, FP64 "
                                          "oracle, single-threaded as the reference (%.1f s, %s PCG iterations)"
                                          % (skip, skip + a.cpu_steps - 1, skip, dt, it_cpu)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
