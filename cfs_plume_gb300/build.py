"""Build libplume.so (CUDA for sm_103a + host C++) in-tree.

    python -m cfs_plume_gb300.build            # library + fluid3D binary
    python -m cfs_plume_gb300.build --oracle   # also the CPU oracle (tests only)

Outputs: cfs_plume_gb300/lib/libplume.so, cfs_plume_gb300/bin/fluid3D,
objects under cfs_plume_gb300/_build/.  Translation units compile in parallel.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
BIN = os.path.join(HERE, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _zlib():
    """(cflags, ldflags) for zlib, or ([], []) when its header is absent (the
    state writer then emits stored gzip blocks)."""
    if not os.path.exists("/usr/include/zlib.h"):
        return [], []
    for d in ("/usr/lib/aarch64-linux-gnu", "/usr/lib/x86_64-linux-gnu", "/usr/lib64", "/usr/lib",
              "/lib/aarch64-linux-gnu", "/lib/x86_64-linux-gnu"):
        if os.path.exists(os.path.join(d, "libz.so")):
            return ["-DPLUME_HAVE_ZLIB"], ["-lz"]
        so1 = os.path.join(d, "libz.so.1")
        if os.path.exists(so1):
            return ["-DPLUME_HAVE_ZLIB"], [so1]
    return [], []


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, ptxas_info=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    zc, zl = _zlib()
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    common_nv = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
    if ptxas_info:
        common_nv += ["-Xptxas", "-v"]
    units = [
        ("engine_f64.cu", [nvcc] + common_nv + ["-fmad=false"]),
        ("engine_f32.cu", [nvcc] + common_nv),
        ("noalloc.cu", [nvcc] + common_nv + ["-fmad=false"]),
        ("unet.cu", [nvcc] + common_nv),
        ("svd.cu", [nvcc] + common_nv),
        ("reduced.cu", [nvcc] + common_nv),
        ("products.cu", [nvcc] + common_nv),
        ("batched_f32.cu", [nvcc] + common_nv),
        ("batched_f64.cu", [nvcc] + common_nv + ["-fmad=false"]),
        ("plume_api.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-I" + os.path.join(cuda, "include")]),
        ("snapshot.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread"] + zc),
        ("state_read.cpp", ["g++", "-O2", "-std=c++17", "-fPIC"] + zc),
        ("batch.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread"]),
        # the box state must round after every operation on Arm hosts too
        ("box.cpp", ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off"]),
    ]
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        for src, cmd in units:
            s = os.path.join(CSRC, src)
            o = os.path.join(OBJ, src + ".o")
            if _newer(o, [s] + headers) and not ptxas_info:
                continue
            jobs.append(ex.submit(_run, cmd + ["-c", s, "-o", o]))
        logs = [j.result() for j in jobs]
    if verbose or ptxas_info:
        for l in logs:
            if l.strip():
                print(l)
    objs = [os.path.join(OBJ, u[0] + ".o") for u in units]
    lib = os.path.join(LIB, "libplume.so")
    if not _newer(lib, objs):
        _run([nvcc, "-shared"] + ARCH + ["-o", lib] + objs + zl)
    # the fluid3D stage binary (host C++ over the C ABI)
    main_src = os.path.join(CSRC, "fluid3d_main.cpp")
    exe = os.path.join(BIN, "fluid3D")
    if os.path.exists(main_src) and not _newer(exe, [main_src, lib] + headers):
        _run(["g++", "-O2", "-std=c++17", "-o", exe, main_src, "-L" + LIB, "-lplume",
              "-Wl,-rpath,$ORIGIN/../lib"])
    # the svdOutOfCoreMultiple stage binary
    svd_src = os.path.join(CSRC, "svd_main.cpp")
    svd_exe = os.path.join(BIN, "svdOutOfCoreMultiple")
    if os.path.exists(svd_src) and not _newer(svd_exe, [svd_src, lib] + headers):
        _run(["g++", "-O2", "-std=c++17", "-o", svd_exe, svd_src, "-L" + LIB, "-lplume",
              "-Wl,-rpath,$ORIGIN/../lib"])
    # the buildProducts and reduced3D stage binaries
    for src_name, exe_name in (("products_main.cpp", "buildProducts"), ("reduced_main.cpp", "reduced3D")):
        src = os.path.join(CSRC, src_name)
        exe_path = os.path.join(BIN, exe_name)
        if os.path.exists(src) and not _newer(exe_path, [src, lib] + headers):
            _run(["g++", "-O2", "-std=c++17", "-o", exe_path, src, "-L" + LIB, "-lplume",
                  "-Wl,-rpath,$ORIGIN/../lib"])
    return lib


def build_oracle(with_reference=True):
    """CPU oracle (test infrastructure): oracle/_build/libplume_oracle.so, and
    oracle/_ref/ (the reference's own step, SVD and reduced stages) when the
    reference sources are present (PLUME_REFERENCE_DIR, else the location the
    oracle's Makefile names)."""
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", odir, "-j8"])
    if not with_reference:
        return
    ref = os.environ.get("PLUME_REFERENCE_DIR")
    if ref:
        _run(["make", "-s", "-C", odir, "-j8", "ref", "REF=" + ref])
    else:  # the oracle recipe's own location of the reference tree, if present
        _run(["make", "-s", "-C", odir, "-j8", "ref-if-present"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print -Xptxas -v register/smem use")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.v, ptxas_info=a.ptxas))
    if a.oracle:
        build_oracle()


if __name__ == "__main__":
    sys.exit(main())
