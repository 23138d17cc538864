"""ctypes mirror of include/plume.h (structs, enums, defaults).

Kept in one place so the library binding, the tests and bench.py agree on the
struct layout.  The numeric defaults are the reference's
(projects/fluid3D/fluid3D.cpp:313-327, src/integrators/FLUID_3D_MIC.cpp:29-54).
"""
import ctypes as C
import struct

ABI_VERSION = 2

OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_IO, ERR_NOT_CONVERGED, ERR_UNSUPPORTED, ERR_STATE = range(9)

PREC_FP64, PREC_FP32 = 0, 1
CRIT_REFERENCE, CRIT_REL2 = 0, 1
SRC_COLUMN, SRC_BOX, SRC_NONE = 0, 1, 2
WARM_ZERO, WARM_PREVIOUS, WARM_LEARNED = 0, 1, 2
PRECOND_MIC, PRECOND_NET = 0, 1

# plume_field, in the state-file order of FLUID_3D_MIC::writeGz (FLUID_3D_MIC.cpp:1057-1103)
FIELDS = [
    "density", "densityOld", "heat", "heatOld", "pressure", "divergence",
    "velocity", "velocityOld", "force", "vorticity", "preprojection",
    "prediffusion", "preadvection", "cachedQuadratic", "postadvection",
    "cachedPressure", "cachedDivergence", "prevorticity",
]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
# PLUME_F_POST_IOP: only assigned by a moving-box step (include/plume_box.h)
FIELD_ID["postIOP"] = len(FIELDS)
VECTOR_FIELDS = {"velocity", "velocityOld", "force", "vorticity", "preprojection",
                 "prediffusion", "preadvection", "cachedQuadratic", "postadvection",
                 "prevorticity", "postIOP"}

# (double)0.1f: the reference stores `_buoyancy = 0.1f` in a double (FLUID_3D_MIC.cpp:36)
BUOYANCY_REF = struct.unpack("f", struct.pack("f", 0.1))[0]


class PlumeParams(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32),
        ("res", C.c_int32 * 3),
        ("bc", C.c_int32 * 6),
        ("dt", C.c_double),
        ("buoyancy", C.c_double),
        ("vorticity_eps", C.c_double),
        ("damping_w", C.c_double),
        ("mic_tau", C.c_double),
        ("mic_sigma", C.c_double),
        ("source", C.c_int32),
        ("box_lo", C.c_int32 * 3),
        ("box_hi", C.c_int32 * 3),
        ("source_noise", C.c_double),
        ("seed", C.c_uint64),
        ("precision", C.c_int32),
        ("criterion", C.c_int32),
        ("tol", C.c_double),
        ("max_iters", C.c_int32),
        ("warm_start", C.c_int32),
        ("cache_fields", C.c_int32),
        ("device", C.c_int32),
        ("preconditioner", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


class PlumeStepStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("converged", C.c_int32),
        ("fallback", C.c_int32),
        ("launches", C.c_int32),
        ("max_residual", C.c_double),
        ("rel_residual", C.c_double),
        ("rhs_norm", C.c_double),
        ("ms_total", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_forces", C.c_double),
        ("ms_vorticity", C.c_double),
        ("ms_advection", C.c_double),
        ("ms_damping", C.c_double),
        ("ms_divergence", C.c_double),
        ("ms_guess", C.c_double),
        ("ms_gradient", C.c_double),
    ]


# the per-stage device times of plume_step_stats, in step order
STAGES = ("forces", "vorticity", "advection", "damping", "divergence", "guess", "solve", "gradient")


def default_params(**kw):
    """Reference defaults; keyword arguments override fields.

    res/bc/box_lo/box_hi accept sequences.
    """
    p = PlumeParams()
    p.abi_version = ABI_VERSION
    p.res[:] = (48, 64, 48)
    p.bc[:] = (1, 1, 1, 1, 0, 0)   # front, back, left, right, top, bottom
    p.dt = 0.1
    p.buoyancy = BUOYANCY_REF
    p.vorticity_eps = 0.0
    p.damping_w = 0.9
    p.mic_tau = 0.97
    p.mic_sigma = 0.25
    p.source = SRC_COLUMN
    p.source_noise = 0.0
    p.seed = 0
    p.precision = PREC_FP64
    p.criterion = CRIT_REFERENCE
    p.tol = 1e-10
    p.max_iters = 1000
    p.warm_start = WARM_ZERO
    p.cache_fields = 1
    p.device = 0
    for k, v in kw.items():
        if k in ("res", "bc", "box_lo", "box_hi"):
            getattr(p, k)[:] = tuple(int(x) for x in v)
        else:
            setattr(p, k, v)
    return p


def scaled_box(res, lo=(20, 2, 20), hi=(28, 6, 28), base=(48, 64, 48)):
    """The 48x64x48 plume source box x,z in [20,28), y in [2,6) scaled to `res`
    by floor(c * res / base) per axis."""
    lo_s = tuple((lo[i] * res[i]) // base[i] for i in range(3))
    hi_s = tuple((hi[i] * res[i]) // base[i] for i in range(3))
    return lo_s, hi_s


def plume_config(res, precision=PREC_FP32, criterion=CRIT_REL2, tol=1e-6, seed=0, **kw):
    """The synthetic plume of the benchmark configurations: closed box (all six
    walls), box source with +-0.05 seeded noise, buoyancy 1 on temperature,
    vorticity 2."""
    lo, hi = scaled_box(res)
    args = dict(res=res, bc=(1, 1, 1, 1, 1, 1), buoyancy=1.0, vorticity_eps=2.0,
                source=SRC_BOX, box_lo=lo, box_hi=hi, source_noise=0.05, seed=seed,
                precision=precision, criterion=criterion, tol=tol)
    args.update(kw)
    return default_params(**args)


class PlumeBox(C.Structure):
    """plume_box (include/plume_box.h): the state of the reference's BOX."""
    _fields_ = [
        ("center", C.c_double * 3),
        ("original_center", C.c_double * 3),
        ("lengths", C.c_double * 3),
        ("rotation", C.c_double * 9),
        ("theta", C.c_double),
        ("phi", C.c_double),
        ("period", C.c_double),
        ("translation_period", C.c_double),
        ("dt", C.c_double),
    ]


class PlumeProductsInfo(C.Structure):
    """plume_products_info (include/plume_reduced.h)."""
    _fields_ = [
        ("ranks", C.c_int32 * 4),
        ("ms_device", C.c_double),
        ("ms_total", C.c_double),
        ("gflop", C.c_double),
    ]


class PlumeSvdInfo(C.Structure):
    """plume_svd_info (include/plume_svd.h)."""
    _fields_ = [
        ("rows", C.c_int32),
        ("cols", C.c_int32),
        ("kept", C.c_int32),
        ("sweeps", C.c_int32),
        ("ms_qr", C.c_double),
        ("ms_svd", C.c_double),
        ("ms_u", C.c_double),
        ("ms_io", C.c_double),
    ]
