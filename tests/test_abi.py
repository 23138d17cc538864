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


def test_struct_sizes_match_header(tmp_path):
    """The ctypes mirrors in _abi.py against sizeof/offsetof of the C header
    structs, compiled with gcc."""
    import subprocess
    from cfs_plume_gb300.batch import PlumeBatchOptions
    checks = [("plume_params", _abi.PlumeParams, "plume.h"),
              ("plume_step_stats", _abi.PlumeStepStats, "plume.h"),
              ("plume_products_info", _abi.PlumeProductsInfo, "plume_reduced.h"),
              ("plume_batch_options", PlumeBatchOptions, "plume_batch.h")]
    lines = ['#include <stdio.h>', '#include <stddef.h>']
    lines += ['#include "%s"' % h for h in sorted({c[2] for c in checks})]
    lines.append("int main(void) {")
    for cname, ct, _ in checks:
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _t in ct._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines.append("  return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                   check=True).stdout.splitlines())
    for cname, ct, _ in checks:
        assert int(got[cname]) == C.sizeof(ct), cname
        for fname, _t in ct._fields_:
            assert int(got[cname + "." + fname]) == getattr(ct, fname).offset, (cname, fname)


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
