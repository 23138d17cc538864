"""Python binding of libplume (ctypes over include/plume.h).

`FLUID_3D_MIC` mirrors the public surface of the reference class
(src/integrators/FLUID_3D_MIC.h:37-120): construct with the resolution and the
six boundary flags, set `vorticityEps`/`buoyancy`, then per step
`addSmokeColumn()` (or `add_source(step)`), `step()`, `writeGz(path)`,
`appendStreams()`.  Field accessors return NumPy copies in the reference
layout (vector fields as (N, 3) arrays of doubles).

The compute runs in the CUDA library; there is no CPU fallback.  Loading fails
with an error when cfs_plume_gb300/lib/libplume.so has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import PlumeBox, PlumeParams, PlumeProductsInfo, PlumeStepStats, PlumeSvdInfo

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libplume.so")
_lib = None


class PlumeError(RuntimeError):
    def __init__(self, status, detail):
        self.status = status
        super().__init__("plume error %d (%s): %s" % (status, _strerror(status), detail))


def load_library(path=LIB_PATH):
    """Load libplume.so and declare its signatures (idempotent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libplume.so not built (%s); run `python -m cfs_plume_gb300.build`" % path)
    lib = C.CDLL(path)
    H = C.c_void_p
    P = C.POINTER
    sig = {
        "plume_default_params": (None, [P(PlumeParams)]),
        "plume_create": (C.c_int, [P(PlumeParams), P(H)]),
        "plume_destroy": (None, [H]),
        "plume_add_source": (C.c_int, [H, C.c_int32]),
        "plume_step": (C.c_int, [H, P(PlumeStepStats)]),
        "plume_add_source_values": (C.c_int, [H, C.c_void_p, C.c_size_t]),
        "plume_run_timed": (C.c_int, [H, C.c_int32, C.c_int32, P(C.c_double), P(PlumeStepStats)]),
        "plume_run": (C.c_int, [H, C.c_int32, C.c_int32, P(PlumeStepStats)]),
        "plume_download": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "plume_upload": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "plume_download_obstacles": (C.c_int, [H, C.c_void_p, C.c_size_t]),
        "plume_get_info": (C.c_int, [H, P(C.c_int32), P(C.c_int32), P(C.c_double), P(C.c_double)]),
        "plume_write_state": (C.c_int, [H, C.c_char_p]),
        "plume_append_streams": (C.c_int, [H, C.c_char_p]),
        "plume_strerror": (C.c_char_p, [C.c_int]),
        "plume_last_error": (C.c_char_p, [H]),
        "plume_solve_poisson": (C.c_int, [H, C.c_void_p, C.c_void_p, P(PlumeStepStats)]),
        "plume_mic_apply": (C.c_int, [H, C.c_void_p, C.c_void_p, C.c_void_p]),
        "plume_mic_diagonal": (C.c_int, [H, C.c_void_p]),
        "plume_sync": (C.c_int, [H]),
        "plume_profile_sweeps": (C.c_int, [H, C.c_int]),
        "plume_snapshot_async": (C.c_int, [H, C.c_char_p, C.c_int32, C.c_int32]),
        "plume_wait_snapshots": (C.c_int, [H]),
        "plume_sweep_times": (C.c_int, [H, P(C.c_double), P(C.c_int64)]),
        "plume_set_wait_gate": (C.c_int, [H, C.c_int32, C.c_int64]),
        "plume_box_init": (C.c_int, [P(PlumeBox), P(C.c_double), P(C.c_double), C.c_double, C.c_double]),
        "plume_box_spin": (C.c_int, [P(PlumeBox)]),
        "plume_box_translate": (C.c_int, [P(PlumeBox)]),
        "plume_box_inside": (C.c_int, [P(PlumeBox), P(C.c_double), P(C.c_int32)]),
        "plume_box_velocity": (C.c_int, [P(PlumeBox), P(C.c_double), P(C.c_double)]),
        "plume_step_moving_box": (C.c_int, [H, P(PlumeBox), P(PlumeStepStats)]),
        "plume_set_initial_velocity_box": (C.c_int, [H, P(PlumeBox)]),
        "plume_download_iop": (C.c_int, [H, C.c_void_p, C.c_void_p, C.c_size_t]),
        "plume_run_moving_timed": (C.c_int, [H, P(PlumeBox), C.c_int32, C.c_int32, P(C.c_double),
                                             P(PlumeStepStats)]),
        "plume_box_stomp_times": (C.c_int, [H, P(C.c_double), P(C.c_int64)]),
        "plume_svd_stream": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_double, C.c_char_p,
                                       C.c_char_p, C.c_int32, P(PlumeSvdInfo)]),
        "plume_svd_columns": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                        C.c_void_p, C.c_void_p, P(C.c_int32), P(PlumeSvdInfo)]),
        "plume_svd_verify": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.c_void_p]),
        "plume_reduced_create": (C.c_int, [H, C.c_char_p, P(H)]),
        "plume_reduced_destroy": (None, [H]),
        "plume_reduced_step": (C.c_int, [H, P(PlumeStepStats)]),
        "plume_reduced_qdot": (C.c_int, [H, C.c_void_p, C.c_int32, P(C.c_int32)]),
        "plume_reduced_dims": (C.c_int, [H, P(C.c_int32)]),
        "plume_reduced_build_products": (C.c_int, [H, C.c_char_p, P(PlumeProductsInfo)]),
        "plume_reduced_set_ground_truth": (C.c_int, [H, C.c_char_p]),
        "plume_reduced_errors": (C.c_int, [H, C.c_void_p, C.c_int32, P(C.c_int32)]),
        "plume_state_read_field": (C.c_int, [C.c_char_p, C.c_int32, C.c_void_p, C.c_size_t, P(C.c_int32)]),
        "plume_state_read_header": (C.c_int, [C.c_char_p, P(C.c_int32), P(C.c_double)]),
        "plume_read_state": (C.c_int, [H, C.c_char_p]),
        "plume_peeled_errors": (C.c_int, [P(C.c_int32), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          P(C.c_double)]),
        "plume_snapshots_create": (C.c_int, [H, C.c_int32, C.c_int32, P(H)]),
        "plume_snapshots_destroy": (None, [H]),
        "plume_snapshots_append": (C.c_int, [H, P(C.c_int32)]),
        "plume_snapshots_dims": (C.c_int, [H, P(C.c_int32), P(C.c_int32)]),
        "plume_snapshots_download": (C.c_int, [H, C.c_void_p, C.c_size_t]),
        "plume_snapshots_svd": (C.c_int, [H, C.c_double, C.c_char_p, C.c_char_p, C.c_void_p,
                                          P(C.c_int32), P(PlumeSvdInfo)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _strerror(status):
    try:
        return load_library().plume_strerror(status).decode()
    except Exception:  # library not loadable: plain number
        return str(status)


def _check(rc, handle=None):
    if rc != 0:
        detail = load_library().plume_last_error(handle).decode(errors="replace")
        raise PlumeError(rc, detail)


class Plume:
    """One simulation on one GPU (a plume_handle)."""

    def __init__(self, params: PlumeParams):
        self.lib = load_library()
        self.params = params
        h = C.c_void_p()
        _check(self.lib.plume_create(C.byref(params), C.byref(h)))
        self.h = h
        self.res = tuple(params.res)
        self.N = self.res[0] * self.res[1] * self.res[2]

    def close(self):
        if getattr(self, "h", None):
            self.lib.plume_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_source(self, step_index):
        _check(self.lib.plume_add_source(self.h, step_index), self.h)

    def add_source_values(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(self.lib.plume_add_source_values(self.h, v.ctypes.data, v.size), self.h)

    def run_timed(self, first_step, n, stats=True):
        """n steps between CUDA events on the handle's stream: (ms, stats)."""
        ms = C.c_double()
        arr = (PlumeStepStats * n)() if stats else None
        _check(self.lib.plume_run_timed(self.h, first_step, n, C.byref(ms), arr), self.h)
        return ms.value, (list(arr) if stats else None)

    def step(self, stats=True):
        st = PlumeStepStats()
        _check(self.lib.plume_step(self.h, C.byref(st) if stats else None), self.h)
        return st if stats else None

    def run(self, first_step, n, stats=False):
        arr = (PlumeStepStats * n)() if stats else None
        _check(self.lib.plume_run(self.h, first_step, n, arr), self.h)
        return list(arr) if stats else None

    def field(self, name):
        fid = _abi.FIELD_ID[name]
        vec = name in _abi.VECTOR_FIELDS
        a = np.empty(3 * self.N if vec else self.N, dtype=np.float64)
        _check(self.lib.plume_download(self.h, fid, a.ctypes.data, a.size), self.h)
        return a

    def read_state(self, path):
        """FLUID_3D_MIC::readGz into this plume (plume_read_state): restores
        the fields and step count of a state file of the same grid and
        parameters, so that stepping continues the run that wrote it."""
        _check(self.lib.plume_read_state(self.h, os.fsencode(path)), self.h)

    def set_field(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        _check(self.lib.plume_upload(self.h, _abi.FIELD_ID[name], a.ctypes.data, a.size), self.h)

    def obstacles(self):
        a = np.empty(self.N, dtype=np.uint8)
        _check(self.lib.plume_download_obstacles(self.h, a.ctypes.data, a.size), self.h)
        return a

    def info(self):
        res = (C.c_int32 * 3)()
        ts, tt, dx = C.c_int32(), C.c_double(), C.c_double()
        _check(self.lib.plume_get_info(self.h, res, C.byref(ts), C.byref(tt), C.byref(dx)), self.h)
        return dict(res=tuple(res), total_steps=ts.value, total_time=tt.value, dx=dx.value)

    def write_state(self, path):
        _check(self.lib.plume_write_state(self.h, os.fsencode(path)), self.h)

    def append_streams(self, directory):
        d = directory if directory.endswith("/") else directory + "/"
        _check(self.lib.plume_append_streams(self.h, os.fsencode(d)), self.h)

    def snapshot_async(self, directory, step, state=True, streams=True):
        """State file and/or stream rows written by the handle's writer thread."""
        d = directory if directory.endswith("/") else directory + "/"
        what = (1 if state else 0) | (2 if streams else 0)
        _check(self.lib.plume_snapshot_async(self.h, os.fsencode(d), step, what), self.h)

    def wait_snapshots(self):
        _check(self.lib.plume_wait_snapshots(self.h), self.h)

    def sync(self):
        """Wait for the handle's stream (plume_sync)."""
        _check(self.lib.plume_sync(self.h), self.h)

    def solve_poisson(self, b, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        st = PlumeStepStats()
        _check(self.lib.plume_solve_poisson(self.h, b.ctypes.data, x.ctypes.data, C.byref(st)), self.h)
        return x, st

    def mic_apply(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.N)
        q = np.zeros(self.N)
        _check(self.lib.plume_mic_apply(self.h, r.ctypes.data, z.ctypes.data, q.ctypes.data), self.h)
        return z, q

    def profile_sweeps(self, on=True):
        """Start (clearing the totals) or stop CUDA-event timing of every MIC sweep launch."""
        _check(self.lib.plume_profile_sweeps(self.h, 1 if on else 0), self.h)

    def sweep_times(self):
        """(summed device ms, number of timed sweep launches) since profiling started."""
        ms, n = C.c_double(), C.c_int64()
        _check(self.lib.plume_sweep_times(self.h, C.byref(ms), C.byref(n)), self.h)
        return ms.value, n.value

    def set_wait_gate(self, closed, poll_limit=1000):
        """Test hook of the MIC sweeps' bounded waits (plume_set_wait_gate):
        closed=True makes every later sweep time out at its entry gate."""
        _check(self.lib.plume_set_wait_gate(self.h, 1 if closed else 0, int(poll_limit)), self.h)

    def mic_diagonal(self):
        p = np.zeros(self.N)
        _check(self.lib.plume_mic_diagonal(self.h, p.ctypes.data), self.h)
        return p

    def step_moving_box(self, box, stats=True):
        """One stepWithMovingObstacle with `box` (a BOX or PlumeBox) as it is."""
        st = PlumeStepStats()
        b = box.state if isinstance(box, BOX) else box
        _check(self.lib.plume_step_moving_box(self.h, C.byref(b), C.byref(st) if stats else None), self.h)
        return st if stats else None

    def set_initial_velocity_box(self, box):
        b = box.state if isinstance(box, BOX) else box
        _check(self.lib.plume_set_initial_velocity_box(self.h, C.byref(b)), self.h)

    def run_moving_timed(self, box, first_step, n, stats=True):
        """n moving steps (source, step, box spin + translate), device-timed:
        (ms, [stats])."""
        b = box.state if isinstance(box, BOX) else box
        arr = (PlumeStepStats * n)() if stats else None
        ms = C.c_double()
        _check(self.lib.plume_run_moving_timed(self.h, C.byref(b), first_step, n, C.byref(ms), arr),
               self.h)
        return ms.value, (list(arr) if stats else None)

    def stomp_times(self):
        """(summed device ms, launches) of the obstacle stomp while sweep profiling is on."""
        ms, n = C.c_double(), C.c_int64()
        _check(self.lib.plume_box_stomp_times(self.h, C.byref(ms), C.byref(n)), self.h)
        return ms.value, n.value

    def iop(self):
        """(inside mask [N] uint8, last-column values [N, 3]) of the last moving step."""
        inside = np.empty(self.N, dtype=np.uint8)
        vals = np.empty(3 * self.N)
        _check(self.lib.plume_download_iop(self.h, inside.ctypes.data, vals.ctypes.data, self.N), self.h)
        return inside, vals.reshape(-1, 3)


class BOX:
    """The reference's moving box (src/geometry/BOX.h) over plume_box."""

    def __init__(self, center, lengths, period, translationPeriod):
        self.lib = load_library()
        self.state = PlumeBox()
        c = (C.c_double * 3)(*center)
        l = (C.c_double * 3)(*lengths)
        _check(self.lib.plume_box_init(C.byref(self.state), c, l, period, translationPeriod))

    def set_dt(self, dt):
        self.state.dt = dt

    def spin(self):
        _check(self.lib.plume_box_spin(C.byref(self.state)))

    def translate_center(self):
        _check(self.lib.plume_box_translate(C.byref(self.state)))

    def inside(self, point):
        out = C.c_int32()
        _check(self.lib.plume_box_inside(C.byref(self.state), (C.c_double * 3)(*point), C.byref(out)))
        return bool(out.value)

    def velocity_at(self, point):
        v = (C.c_double * 3)()
        _check(self.lib.plume_box_velocity(C.byref(self.state), (C.c_double * 3)(*point), v))
        return tuple(v)

    @property
    def theta(self):
        return self.state.theta

    @property
    def phi(self):
        return self.state.phi

    @property
    def center(self):
        return tuple(self.state.center)


class FLUID_3D_MIC:
    """Facade with the reference class's names (FLUID_3D_MIC.h:37-120).

    The device state is created on first use so that `vorticityEps` and
    `buoyancy` can be assigned after construction, as fluid3D.cpp:346 does.
    """

    def __init__(self, xRes, yRes, zRes, amplify=4, boundaries=None, **params):
        kw = dict(res=(xRes, yRes, zRes))
        if boundaries is not None:
            kw["bc"] = tuple(boundaries)
        kw.update(params)
        self._params = _abi.default_params(**kw)
        self._plume = None
        self._source_step = 0
        self.snapshotPath = ""

    # reference accessors that are assignable (Real& vorticityEps(), buoyancy())
    @property
    def vorticityEps(self):
        return self._params.vorticity_eps

    @vorticityEps.setter
    def vorticityEps(self, v):
        self._require_fresh()
        self._params.vorticity_eps = float(v)

    @property
    def buoyancy(self):
        return self._params.buoyancy

    @buoyancy.setter
    def buoyancy(self, v):
        self._require_fresh()
        self._params.buoyancy = float(v)

    def _require_fresh(self):
        if self._plume is not None:
            raise RuntimeError("parameters must be set before the first step")

    @property
    def plume(self):
        if self._plume is None:
            self._plume = Plume(self._params)
        return self._plume

    def xRes(self):
        return self._params.res[0]

    def yRes(self):
        return self._params.res[1]

    def zRes(self):
        return self._params.res[2]

    def dx(self):
        return self.plume.info()["dx"]

    def addSmokeColumn(self):
        self.plume.add_source(self._source_step)
        self._source_step += 1

    def step(self):
        return self.plume.step()

    def stepWithMovingObstacle(self, box):
        return self.plume.step_moving_box(box)

    def setInitialVelocity(self, box):
        self.plume.set_initial_velocity_box(box)

    def writeGz(self, filename):
        self.plume.write_state(filename)

    def readGz(self, filename):
        self.plume.read_state(filename)

    def appendStreams(self):
        if not self.snapshotPath:
            raise RuntimeError("snapshotPath is empty")
        self.plume.append_streams(self.snapshotPath)

    def _vec(self, name):
        return self.plume.field(name).reshape(-1, 3)

    def velocity(self):
        return self._vec("velocity")

    def velocityOld(self):
        return self._vec("velocityOld")

    def force(self):
        return self._vec("force")

    def vorticity(self):
        return self._vec("vorticity")

    def density(self):
        return self.plume.field("density")

    def pressure(self):
        return self.plume.field("pressure")

    def divergence(self):
        return self.plume.field("divergence")

    def preprojection(self):
        return self._vec("preprojection")

    def prediffusion(self):
        return self._vec("prediffusion")

    def prevorticity(self):
        return self._vec("prevorticity")

    def preadvection(self):
        return self._vec("preadvection")

    def postadvection(self):
        return self._vec("postadvection")

    def cachedQuadratic(self):
        return self._vec("cachedQuadratic")

    def cachedPressure(self):
        return self.plume.field("cachedPressure")

    def cachedDivergence(self):
        return self.plume.field("cachedDivergence")

    def postIOP(self):
        return self._vec("postIOP")


def svd_stream(prefix, reduced_path, scratch_path, discard_threshold=1e-9, u_path=None, pca_path=None,
               device=0):
    """BIG_MATRIX::outOfCoreSVD + writeFinalU for one snapshot stream on the GPU
    (include/plume_svd.h).  Returns the plume_svd_info as a dict."""
    lib = load_library()
    info = PlumeSvdInfo()
    enc = lambda v: None if v is None else os.fsencode(v)
    _check(lib.plume_svd_stream(enc(prefix), enc(reduced_path), enc(scratch_path), discard_threshold,
                                enc(u_path), enc(pca_path), device, C.byref(info)))
    return {k: getattr(info, k) for k, _ in PlumeSvdInfo._fields_}


def svd_columns(A, discard_threshold=1e-9, with_u=True, device=0):
    """Snapshot SVD of A (n x m, one snapshot per column) on the GPU:
    (pca values [m], kept, U [n x kept] or None, info dict)."""
    lib = load_library()
    A = np.asfortranarray(A, dtype=np.float64)
    n, m = A.shape
    pca = np.empty(m)
    U = np.empty((n, m), order="F") if with_u else None
    kept = C.c_int32()
    info = PlumeSvdInfo()
    _check(lib.plume_svd_columns(A.ctypes.data, n, m, discard_threshold, device, pca.ctypes.data,
                                 U.ctypes.data if with_u else None, C.byref(kept), C.byref(info)))
    k = kept.value
    return pca, k, (U[:, :k].copy() if with_u else None), {f: getattr(info, f) for f, _ in PlumeSvdInfo._fields_}


def svd_verify(prefix, u_path, count=10, device=0):
    """|c - U U^T c| for the first `count` snapshots of the stream (verifyResults)."""
    lib = load_library()
    d = np.empty(count)
    _check(lib.plume_svd_verify(os.fsencode(prefix), os.fsencode(u_path), count, device, d.ctypes.data))
    return d


STREAMS = {"final": 0, "preproject": 1, "prediffuse": 2, "preadvect": 3, "iop": 4, "pressure": 5}


class Snapshots:
    """Rows of one appendStreams stream kept in device memory
    (plume_snapshots, include/plume_svd.h)."""

    def __init__(self, plume, stream, capacity):
        self.h = None
        self.lib = load_library()
        self.plume = plume
        h = C.c_void_p()
        _check(self.lib.plume_snapshots_create(plume.h, STREAMS[stream], capacity, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.plume_snapshots_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def append(self):
        n = C.c_int32()
        _check(self.lib.plume_snapshots_append(self.h, C.byref(n)))
        return n.value

    def dims(self):
        r, c = C.c_int32(), C.c_int32()
        _check(self.lib.plume_snapshots_dims(self.h, C.byref(r), C.byref(c)))
        return r.value, c.value

    def rows(self):
        r, c = self.dims()
        a = np.empty((r, c))
        _check(self.lib.plume_snapshots_download(self.h, a.ctypes.data, a.size))
        return a

    def svd(self, discard_threshold=1e-9, u_path=None, pca_path=None):
        """Factor the held rows (consumed): (pca values, kept, info dict)."""
        r, _ = self.dims()
        pca = np.empty(max(r, 1))
        kept = C.c_int32()
        info = PlumeSvdInfo()
        enc = lambda v: None if v is None else os.fsencode(v)
        _check(self.lib.plume_snapshots_svd(self.h, discard_threshold, enc(u_path), enc(pca_path),
                                            pca.ctypes.data, C.byref(kept), C.byref(info)))
        return pca[:r], kept.value, {f: getattr(info, f) for f, _ in PlumeSvdInfo._fields_}


def read_state_field(path, name):
    """FLUID_3D_MIC::readGz for one field of a state file, on the host
    (plume_state_read_field): (values, res) with the values as float64 in
    the reference layout (N, or 3N interleaved for vector fields)."""
    lib = load_library()
    res = (C.c_int32 * 3)()
    _check(lib.plume_state_read_field(os.fsencode(path), 0, None, 0, res))
    N = res[0] * res[1] * res[2]
    a = np.empty(3 * N if name in _abi.VECTOR_FIELDS else N, dtype=np.float64)
    _check(lib.plume_state_read_field(os.fsencode(path), _abi.FIELD_ID[name], a.ctypes.data, a.size, None))
    return a, tuple(res)


def peeled_errors(res, velocity, density, truth_velocity, truth_density):
    """diffGroundTruth's norms (plume_peeled_errors): velocity abs, velocity
    relative, density abs, density relative over the interior cells."""
    lib = load_library()
    arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel()
            for a in (velocity, density, truth_velocity, truth_density)]
    N = int(res[0]) * int(res[1]) * int(res[2])
    if arrs[0].size != 3 * N or arrs[2].size != 3 * N or arrs[1].size != N or arrs[3].size != N:
        raise ValueError("fields do not match the grid")
    r = (C.c_int32 * 3)(*[int(v) for v in res])
    out = (C.c_double * 4)()
    _check(lib.plume_peeled_errors(r, *[a.ctypes.data for a in arrs], out))
    return np.array(list(out))


def build_products(plume, reduced_path):
    """The projected operators of a reduced model for the plume's grid and
    walls (plume_reduced_build_products, include/plume_reduced.h; the
    reference's buildOutOfCoreMatrices run by buildProducts): reads
    U.pressure, U.preproject, U.prediffuse and U.final under reduced_path and
    writes projected.A, projected.vtod, damping.peeled, projected.ptof,
    projected.ptov and inverseProduct there.  Returns the plume_products_info
    as a dict."""
    lib = load_library()
    d = reduced_path if reduced_path.endswith("/") else reduced_path + "/"
    info = PlumeProductsInfo()
    _check(lib.plume_reduced_build_products(plume.h, os.fsencode(d), C.byref(info)))
    return dict(ranks=tuple(info.ranks), ms_device=info.ms_device, ms_total=info.ms_total, gflop=info.gflop)


class ReducedModel:
    """A reduced (subspace) model attached to a plume handle
    (plume_reduced, include/plume_reduced.h): step() is the reference's
    stepReorderedCubatureStam on the handle's state.  Creating it builds the
    projected operators first when they are missing or stale, as the
    reference's constructor does."""

    def __init__(self, plume, reduced_path):
        self.h = None
        self.lib = load_library()
        self.plume = plume
        d = reduced_path if reduced_path.endswith("/") else reduced_path + "/"
        h = C.c_void_p()
        _check(self.lib.plume_reduced_create(plume.h, os.fsencode(d), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.plume_reduced_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def step(self, stats=True):
        st = PlumeStepStats()
        _check(self.lib.plume_reduced_step(self.h, C.byref(st) if stats else None))
        return st if stats else None

    def qdot(self):
        n = C.c_int32()
        _check(self.lib.plume_reduced_qdot(self.h, None, 0, C.byref(n)))
        q = np.empty(n.value)
        _check(self.lib.plume_reduced_qdot(self.h, q.ctypes.data, n.value, C.byref(n)))
        return q

    def set_ground_truth(self, full_rank_path):
        """diffGroundTruth after every step against <path>fluid.%04i.fluid3d.gz
        (plume_reduced_set_ground_truth); None turns it off."""
        p = None if not full_rank_path else os.fsencode(full_rank_path)
        _check(self.lib.plume_reduced_set_ground_truth(self.h, p))

    def errors(self):
        """The recorded ground-truth errors, one row per compared step:
        velocity abs, velocity relative, density abs, density relative."""
        n = C.c_int32()
        _check(self.lib.plume_reduced_errors(self.h, None, 0, C.byref(n)))
        out = np.empty((n.value, 4))
        if n.value:
            _check(self.lib.plume_reduced_errors(self.h, out.ctypes.data, out.size, C.byref(n)))
        return out

    def dims(self):
        d = (C.c_int32 * 5)()
        _check(self.lib.plume_reduced_dims(self.h, d))
        return dict(preadvect=d[0], prediffuse=d[1], preproject=d[2], final=d[3], cubature_points=d[4])
