"""Python binding of many independent plumes on one GPU (include/plume_batch.h).

Two engines: "fused" (one launch per stage over every plume, each step one
CUDA graph launch, tile shapes from the autotuner) and "streams" (one
plume_handle and CUDA stream per plume, stepped from host threads)."""
import ctypes as C
import json

import numpy as np

from . import _abi
from .plume import PlumeError, PlumeStepStats, load_library

ENGINE_FUSED = 0
ENGINE_STREAMS = 1
ENGINES = {"fused": ENGINE_FUSED, "streams": ENGINE_STREAMS}


class PlumeBatchOptions(C.Structure):
    _fields_ = [
        ("engine", C.c_int32),
        ("graph", C.c_int32),
        ("tune", C.c_int32),
        ("groups", C.c_int32),
        ("tune_cache", C.c_char_p),
        ("persistent", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


_signed = False


def _lib():
    global _signed
    lib = load_library()
    if not _signed:
        V, P = C.c_void_p, C.POINTER
        sig = {
            "plume_batch_params": (C.c_int, [C.c_uint64, C.c_int32, P(_abi.PlumeParams)]),
            "plume_batch_default_options": (None, [P(PlumeBatchOptions)]),
            "plume_batch_create": (C.c_int, [P(_abi.PlumeParams), C.c_int32, P(V)]),
            "plume_batch_create_ex": (C.c_int, [P(_abi.PlumeParams), C.c_int32, P(PlumeBatchOptions), P(V)]),
            "plume_batch_destroy": (None, [V]),
            "plume_batch_size": (C.c_int, [V, P(C.c_int32)]),
            "plume_batch_handle": (C.c_int, [V, C.c_int32, P(V)]),
            "plume_batch_download": (C.c_int, [V, C.c_int32, C.c_int32, V, C.c_size_t]),
            "plume_batch_tuning": (C.c_int, [V, C.c_char_p, C.c_size_t, P(C.c_size_t)]),
            "plume_batch_run": (C.c_int, [V, C.c_int32, C.c_int32, C.c_int32, P(C.c_double), V]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _signed = True
    return lib


def _check(rc):
    if rc != 0:
        raise PlumeError(rc, load_library().plume_last_error(None).decode())


def batch_params(seed, index):
    """Parameters of instance `index` of the batched-plume configuration."""
    p = _abi.PlumeParams()
    _check(_lib().plume_batch_params(seed, index, C.byref(p)))
    return p


def default_options():
    o = PlumeBatchOptions()
    _lib().plume_batch_default_options(C.byref(o))
    return o


class PlumeBatch:
    """n plumes advanced together.  engine: "fused" (default) or "streams";
    graph / tune / tune_cache / groups / persistent: the fused engine's options."""

    def __init__(self, params, engine="fused", graph=True, tune=True, tune_cache=None, groups=0,
                 persistent=False):
        self.lib = _lib()
        arr = (_abi.PlumeParams * len(params))(*params)
        o = default_options()
        o.engine = ENGINES[engine]
        o.graph = 1 if graph else 0
        o.tune = 1 if tune else 0
        o.groups = groups
        o.persistent = 1 if persistent else 0
        self._cache = tune_cache.encode() if tune_cache else None
        o.tune_cache = self._cache
        self.h = C.c_void_p()
        _check(self.lib.plume_batch_create_ex(arr, len(params), C.byref(o), C.byref(self.h)))
        self.n = len(params)
        self.engine = engine
        self.params = list(params)

    def run(self, first_step, steps, threads=0, stats=True):
        """Advance every instance; returns (seconds, stats[instance][step] or None)."""
        secs = C.c_double()
        arr = (PlumeStepStats * (self.n * steps))() if stats else None
        _check(self.lib.plume_batch_run(self.h, first_step, steps, threads, C.byref(secs), arr))
        if not stats:
            return secs.value, None
        return secs.value, [list(arr[i * steps:(i + 1) * steps]) for i in range(self.n)]

    def handle(self, i):
        h = C.c_void_p()
        _check(self.lib.plume_batch_handle(self.h, i, C.byref(h)))
        return h

    def field(self, i, name):
        """Instance i's field as FP64 (vector fields interleaved per cell)."""
        p = self.params[i]
        N = p.res[0] * p.res[1] * p.res[2]
        vec = name in _abi.VECTOR_FIELDS
        a = np.empty(3 * N if vec else N, dtype=np.float64)
        _check(self.lib.plume_batch_download(self.h, i, _abi.FIELD_ID[name], a.ctypes.data, a.size))
        return a

    def tuning(self):
        """The fused engine's tile shapes (and how they were chosen) as a dict."""
        need = C.c_size_t()
        _check(self.lib.plume_batch_tuning(self.h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value + 1)
        _check(self.lib.plume_batch_tuning(self.h, buf, len(buf), C.byref(need)))
        return json.loads(buf.value.decode())

    def close(self):
        if self.h:
            self.lib.plume_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
