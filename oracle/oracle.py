"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle
(oracle/_build/libplume_oracle.so, built from plume_oracle.cpp by oracle/Makefile).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs, never by the product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from cfs_plume_gb300 import _abi
from cfs_plume_gb300._abi import PlumeBox, PlumeParams, PlumeStepStats

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libplume_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "fluid3d_ref")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = C.CDLL(LIB)
    H = C.c_void_p
    P = C.POINTER
    sig = {
        "orc_create": (H, [P(PlumeParams)]),
        "orc_destroy": (None, [H]),
        "orc_add_source": (None, [H, C.c_int32]),
        "orc_step": (None, [H, P(PlumeStepStats)]),
        "orc_reduced_prestep": (None, [H]),
        "orc_get": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "orc_set": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "orc_get_obstacles": (C.c_int, [H, C.c_void_p, C.c_size_t]),
        "orc_total_steps": (C.c_int32, [H]),
        "orc_mic_precon": (None, [P(C.c_int32), P(C.c_int32), C.c_double, C.c_double, C.c_void_p]),
        "orc_mic_apply": (None, [P(C.c_int32), P(C.c_int32), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "orc_mult_a": (None, [P(C.c_int32), P(C.c_int32), C.c_void_p, C.c_void_p]),
        "orc_advect_scalar": (None, [P(C.c_int32), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
        "orc_solve_poisson": (C.c_int32, [P(PlumeParams), C.c_void_p, C.c_void_p, P(PlumeStepStats)]),
        "orc_source_value": (C.c_double, [C.c_uint64, C.c_int32, C.c_int64, C.c_double]),
        "orc_box_init": (None, [P(PlumeBox), P(C.c_double), P(C.c_double), C.c_double, C.c_double]),
        "orc_box_spin": (None, [P(PlumeBox)]),
        "orc_box_translate": (None, [P(PlumeBox)]),
        "orc_box_inside": (C.c_int, [P(PlumeBox), P(C.c_double)]),
        "orc_box_velocity": (None, [P(PlumeBox), P(C.c_double), P(C.c_double)]),
        "orc_step_moving_box": (None, [H, P(PlumeBox), P(PlumeStepStats)]),
        "orc_set_initial_velocity_box": (None, [H, P(PlumeBox)]),
        "orc_iop_entries": (C.c_int64, [H, P(C.c_int32), C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class Oracle:
    """FP64 CPU restatement of FLUID_3D_MIC, same parameter struct as the product."""

    def __init__(self, params: PlumeParams):
        self.lib = load()
        self.params = params
        self.h = self.lib.orc_create(C.byref(params))
        if not self.h:
            raise ValueError("oracle rejected parameters")
        self.res = tuple(params.res)
        self.N = self.res[0] * self.res[1] * self.res[2]

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_source(self, step):
        self.lib.orc_add_source(self.h, step)

    def step(self):
        st = PlumeStepStats()
        self.lib.orc_step(self.h, C.byref(st))
        return st

    def reduced_prestep(self):
        """The full-space part of the reference's reduced step (buoyancy,
        vorticity, density and heat advection); reduced_oracle.py does the
        rest."""
        self.lib.orc_reduced_prestep(self.h)

    def field(self, name):
        n = 3 * self.N if name in _abi.VECTOR_FIELDS else self.N
        a = np.empty(n)
        assert self.lib.orc_get(self.h, _abi.FIELD_ID[name], a.ctypes.data, n) == 0
        return a

    def set_field(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        assert self.lib.orc_set(self.h, _abi.FIELD_ID[name], a.ctypes.data, a.size) == 0

    def obstacles(self):
        a = np.empty(self.N, dtype=np.uint8)
        assert self.lib.orc_get_obstacles(self.h, a.ctypes.data, a.size) == 0
        return a

    def step_moving_box(self, box):
        st = PlumeStepStats()
        self.lib.orc_step_moving_box(self.h, C.byref(box), C.byref(st))
        return st

    def set_initial_velocity_box(self, box):
        self.lib.orc_set_initial_velocity_box(self.h, C.byref(box))

    def iop_entries(self):
        """((rows, cols), ij [n, 2] int32, values [n]) of the obstacle matrix, or None."""
        rc = (C.c_int32 * 2)()
        n = self.lib.orc_iop_entries(self.h, rc, None, None)
        if n < 0:
            return None
        ij = np.empty((n, 2), dtype=np.int32)
        val = np.empty(n)
        self.lib.orc_iop_entries(self.h, rc, ij.ctypes.data, val.ctypes.data)
        return (rc[0], rc[1]), ij, val


def _arr3(v):
    return (C.c_int32 * len(v))(*v)


def mic_precon(res, bc, tau=0.97, sigma=0.25):
    n = res[0] * res[1] * res[2]
    out = np.zeros(n)
    load().orc_mic_precon(_arr3(res), _arr3(bc), tau, sigma, out.ctypes.data)
    return out


def mic_apply(res, bc, precon, r):
    n = res[0] * res[1] * res[2]
    z, q = np.zeros(n), np.zeros(n)
    r = np.ascontiguousarray(r, dtype=np.float64)
    precon = np.ascontiguousarray(precon, dtype=np.float64)
    load().orc_mic_apply(_arr3(res), _arr3(bc), precon.ctypes.data, r.ctypes.data, z.ctypes.data, q.ctypes.data)
    return z, q


def mult_a(res, bc, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = np.zeros_like(x)
    load().orc_mult_a(_arr3(res), _arr3(bc), x.ctypes.data, b.ctypes.data)
    return b


def solve_poisson(params, b, x0=None):
    n = params.res[0] * params.res[1] * params.res[2]
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    st = PlumeStepStats()
    load().orc_solve_poisson(C.byref(params), x.ctypes.data, b.ctypes.data, C.byref(st))
    return x, st


def source_value(seed, step, cell, noise):
    return load().orc_source_value(seed, step, cell, noise)


def box_init(center, lengths, period, translation_period):
    """BOX(center, lengths, period, translationPeriod) restated (plume_box)."""
    b = PlumeBox()
    load().orc_box_init(C.byref(b), (C.c_double * 3)(*center), (C.c_double * 3)(*lengths),
                        period, translation_period)
    return b


def box_spin(b):
    load().orc_box_spin(C.byref(b))


def box_translate(b):
    load().orc_box_translate(C.byref(b))


def box_inside(b, p):
    return bool(load().orc_box_inside(C.byref(b), (C.c_double * 3)(*p)))


def box_velocity(b, p):
    v = (C.c_double * 3)()
    load().orc_box_velocity(C.byref(b), (C.c_double * 3)(*p), v)
    return tuple(v)
