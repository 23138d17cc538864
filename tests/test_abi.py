"""CPU tests of the C ABI: the library loads, exports every declared entry
point, its defaults are the reference's, and without a usable GPU it fails with
a status code instead of crashing."""
import ctypes as C
import glob
import os
import re

import pytest

from cfs_plume_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(plume_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_core_api():
    names = declared_functions()
    for core in ("plume_create", "plume_step", "plume_download", "plume_write_state",
                 "plume_append_streams", "plume_solve_poisson", "plume_destroy"):
        assert core in names


def test_library_exports_every_declared_symbol(plume_lib):
    missing = [n for n in declared_functions() if not hasattr(plume_lib, n)]
    assert not missing, missing


def test_default_params_are_the_reference_defaults(plume_lib):
    p = _abi.PlumeParams()
    plume_lib.plume_default_params(C.byref(p))
    q = _abi.default_params()
    for name, _ in _abi.PlumeParams._fields_:
        a, b = getattr(p, name), getattr(q, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name
    assert p.buoyancy == float.fromhex("0x1.99999a0000000p-4")  # (double)0.1f


def test_struct_sizes_match_header():
    # plume_params: see include/plume.h; offsets must agree with the C layout
    # (checked against sizeof/offsetof of the C header compiled with gcc)
    assert C.sizeof(_abi.PlumeParams) == 200
    assert _abi.PlumeParams.seed.offset == 128
    assert C.sizeof(_abi.PlumeStepStats) == 56
    assert C.sizeof(_abi.PlumeProductsInfo) == 40


def test_invalid_params_are_rejected_without_a_device(plume_lib):
    from cfs_plume_gb300 import plume
    p = _abi.default_params(res=(3, 64, 48))
    with pytest.raises(plume.PlumeError) as e:
        plume.Plume(p)
    assert e.value.status in (_abi.ERR_INVALID, _abi.ERR_CUDA)
    p = _abi.default_params(abi_version=99)
    with pytest.raises(plume.PlumeError) as e:
        plume.Plume(p)
    assert e.value.status == _abi.ERR_INVALID


def test_strerror_covers_every_status(plume_lib):
    texts = {plume_lib.plume_strerror(s).decode() for s in range(9)}
    assert len(texts) == 9
