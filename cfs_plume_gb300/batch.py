"""Python binding of many independent plumes on one GPU (include/plume_batch.h)."""
import ctypes as C

from . import _abi
from .plume import PlumeError, PlumeStepStats, load_library

_signed = False


def _lib():
    global _signed
    lib = load_library()
    if not _signed:
        V, P = C.c_void_p, C.POINTER
        sig = {
            "plume_batch_params": (C.c_int, [C.c_uint64, C.c_int32, P(_abi.PlumeParams)]),
            "plume_batch_create": (C.c_int, [P(_abi.PlumeParams), C.c_int32, P(V)]),
            "plume_batch_destroy": (None, [V]),
            "plume_batch_size": (C.c_int, [V, P(C.c_int32)]),
            "plume_batch_handle": (C.c_int, [V, C.c_int32, P(V)]),
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


class PlumeBatch:
    def __init__(self, params):
        self.lib = _lib()
        arr = (_abi.PlumeParams * len(params))(*params)
        self.h = C.c_void_p()
        _check(self.lib.plume_batch_create(arr, len(params), C.byref(self.h)))
        self.n = len(params)
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

    def close(self):
        if self.h:
            self.lib.plume_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
