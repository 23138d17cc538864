"""Python binding of the learned warm start (include/plume_net.h) over ctypes.

The network, its pair store and its trainer all run on the GPU inside
libplume; this module only moves host buffers and checks status codes.
"""
import ctypes as C
import os

import numpy as np

from .plume import PlumeError, load_library

_signed = False
LOSS_MSE, LOSS_ENERGY = 0, 1
PAIRS_SOLVE, PAIRS_CORRECTION, PAIRS_ITERATE = 0, 1, 2


class PlumeDatasetSpec(C.Structure):
    _fields_ = [("res", C.c_int32 * 3), ("plumes", C.c_int32), ("steps", C.c_int32), ("skip", C.c_int32),
                ("threads", C.c_int32), ("device", C.c_int32), ("seed", C.c_uint64), ("tol", C.c_double),
                ("kind", C.c_int32)]


class PlumeTrainSpec(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("val_pairs", C.c_int32), ("loss", C.c_int32),
                ("lr", C.c_float), ("lr_final", C.c_float), ("seed", C.c_uint64)]


def _lib():
    global _signed
    lib = load_library()
    if not _signed:
        V, P = C.c_void_p, C.POINTER
        sig = {
            "plume_net_create": (C.c_int, [C.c_uint64, C.c_int32, P(V)]),
            "plume_net_destroy": (None, [V]),
            "plume_net_num_params": (C.c_int, [V, P(C.c_int64)]),
            "plume_net_get_params": (C.c_int, [V, V, C.c_int64]),
            "plume_net_set_params": (C.c_int, [V, V, C.c_int64]),
            "plume_net_get_scale": (C.c_int, [V, P(C.c_float)]),
            "plume_net_set_scale": (C.c_int, [V, C.c_float]),
            "plume_net_save": (C.c_int, [V, C.c_char_p]),
            "plume_net_load": (C.c_int, [V, C.c_char_p]),
            "plume_net_forward": (C.c_int, [V, P(C.c_int32), C.c_int32, V, V]),
            "plume_net_loss_grad": (C.c_int, [V, P(C.c_int32), C.c_int32, C.c_int32, V, V, P(C.c_double), V]),
            "plume_dataset_generate": (C.c_int, [P(PlumeDatasetSpec), P(V)]),
            "plume_dataset_destroy": (None, [V]),
            "plume_dataset_info": (C.c_int, [V, P(C.c_int32), P(C.c_double), P(C.c_double)]),
            "plume_dataset_get_pair": (C.c_int, [V, C.c_int32, V, V]),
            "plume_net_train": (C.c_int, [V, V, P(PlumeTrainSpec), V, V, P(C.c_double)]),
            "plume_attach_net": (C.c_int, [V, V]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _signed = True
    return lib


def _check(rc):
    if rc != 0:
        lib = load_library()
        raise PlumeError(rc, lib.plume_last_error(None).decode())


def _res(res):
    return (C.c_int32 * 3)(*[int(v) for v in res])


class PlumeNet:
    """The warm-start U-Net (3 levels, 16/32/64 channels, BF16 tensor-core kernels)."""

    def __init__(self, seed=0, device=0, path=None):
        self.lib = _lib()
        self.h = C.c_void_p()
        _check(self.lib.plume_net_create(seed, device, C.byref(self.h)))
        n = C.c_int64()
        _check(self.lib.plume_net_num_params(self.h, C.byref(n)))
        self.num_params = n.value
        if path is not None:
            self.load(path)

    def close(self):
        if self.h:
            self.lib.plume_net_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        a = np.empty(self.num_params, dtype=np.float32)
        _check(self.lib.plume_net_get_params(self.h, a.ctypes.data, a.size))
        return a

    @params.setter
    def params(self, values):
        a = np.ascontiguousarray(values, dtype=np.float32)
        _check(self.lib.plume_net_set_params(self.h, a.ctypes.data, a.size))

    @property
    def scale(self):
        s = C.c_float()
        _check(self.lib.plume_net_get_scale(self.h, C.byref(s)))
        return s.value

    @scale.setter
    def scale(self, value):
        _check(self.lib.plume_net_set_scale(self.h, float(value)))

    def save(self, path):
        _check(self.lib.plume_net_save(self.h, os.fsencode(path)))

    def load(self, path):
        _check(self.lib.plume_net_load(self.h, os.fsencode(path)))

    def forward(self, inp, res):
        inp = np.ascontiguousarray(inp, dtype=np.float32)
        batch = inp.size // int(np.prod(res))
        out = np.empty_like(inp)
        _check(self.lib.plume_net_forward(self.h, _res(res), batch, inp.ctypes.data, out.ctypes.data))
        return out

    def loss_grad(self, inp, tgt, res, loss=LOSS_MSE):
        inp = np.ascontiguousarray(inp, dtype=np.float32)
        tgt = np.ascontiguousarray(tgt, dtype=np.float32)
        batch = inp.size // int(np.prod(res))
        value = C.c_double()
        grad = np.empty(self.num_params, dtype=np.float32)
        _check(self.lib.plume_net_loss_grad(self.h, _res(res), batch, int(loss), inp.ctypes.data,
                                            tgt.ctypes.data, C.byref(value), grad.ctypes.data))
        return value.value, grad

    def train(self, dataset, epochs=1, batch=4, val_pairs=0, lr=1e-3, lr_final=1e-4, seed=0, loss=LOSS_ENERGY):
        sp = PlumeTrainSpec(epochs=epochs, batch=batch, val_pairs=val_pairs, loss=loss, lr=lr,
                            lr_final=lr_final, seed=seed)
        tl = np.zeros(epochs, dtype=np.float32)
        vl = np.zeros(epochs, dtype=np.float32)
        secs = C.c_double()
        _check(self.lib.plume_net_train(self.h, dataset.h, C.byref(sp), tl.ctypes.data, vl.ctypes.data,
                                        C.byref(secs)))
        return tl, vl, secs.value

    def attach(self, plume):
        """Use this network for the PLUME_WARM_LEARNED solves of a Plume handle."""
        rc = self.lib.plume_attach_net(plume.h, self.h)
        if rc != 0:
            raise PlumeError(rc, self.lib.plume_last_error(None).decode())


class PairStore:
    """(b / rms(b), p / rms(b)) pairs from plain solves of randomised plumes, on the GPU."""

    def __init__(self, res, plumes, steps, skip=0, threads=8, seed=0, tol=1e-6, device=0, kind=PAIRS_SOLVE):
        self.lib = _lib()
        self.res = tuple(res)
        sp = PlumeDatasetSpec(res=(C.c_int32 * 3)(*res), plumes=plumes, steps=steps, skip=skip, threads=threads,
                              device=device, seed=seed, tol=tol, kind=kind)
        self.h = C.c_void_p()
        _check(self.lib.plume_dataset_generate(C.byref(sp), C.byref(self.h)))
        n, rms, secs = C.c_int32(), C.c_double(), C.c_double()
        _check(self.lib.plume_dataset_info(self.h, C.byref(n), C.byref(rms), C.byref(secs)))
        self.pairs, self.target_rms, self.seconds = n.value, rms.value, secs.value

    def pair(self, i):
        N = int(np.prod(self.res))
        a = np.empty(N, dtype=np.float32)
        b = np.empty(N, dtype=np.float32)
        _check(self.lib.plume_dataset_get_pair(self.h, i, a.ctypes.data, b.ctypes.data))
        return a, b

    def close(self):
        if self.h:
            self.lib.plume_dataset_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
