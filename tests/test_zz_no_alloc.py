"""plume_mic_apply_noalloc (include/plume_noalloc.h): the MIC(0) apply whose
work vectors live in a fixed device array, against the allocating
plume_mic_apply (FLUID_3D_MIC::applyMICPreconditioner, FLUID_3D_MIC.cpp:864-899)
on the same grid.  Kept in a file collected last so that it also runs after
every other GPU test in the same process."""
import ctypes

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from cfs_plume_gb300.plume import Plume, load_library

PLUME_OK = 0
PLUME_ERR_INVALID = 1


def _noalloc(lib):
    f = lib.plume_mic_apply_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _ints(vals):
    return (ctypes.c_int32 * len(vals))(*vals)


def test_oversize_grid_is_rejected_before_any_device_work():
    f = _noalloc(load_library())
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    bc = _ints([1] * 6)
    # 130 x 200 x 130 needs 128 * 229 * 128 skewed values, above the fixed scratch
    assert f(_ints([130, 200, 130]), bc, fake, fake, fake, None) == PLUME_ERR_INVALID
    # x above 258 cells is outside the sweep kernels' row width
    assert f(_ints([300, 6, 6]), bc, fake, fake, fake, None) == PLUME_ERR_INVALID
    assert f(_ints([16, 3, 16]), bc, fake, fake, fake, None) == PLUME_ERR_INVALID
    assert f(_ints([16, 16, 16]), _ints([1, 1, 2, 1, 1, 1]), fake, fake, fake, None) == PLUME_ERR_INVALID
    assert f(_ints([16, 16, 16]), bc, None, fake, fake, None) == PLUME_ERR_INVALID
    # sizes whose skewed vector overflows 32-bit arithmetic are refused too
    assert f(_ints([258, 100000, 100000]), bc, fake, fake, fake, None) == PLUME_ERR_INVALID
    assert f(_ints([258, 2 ** 31 - 1, 1000]), bc, fake, fake, fake, None) == PLUME_ERR_INVALID


def _call(f, torch, dev, res, bc, d_pre, r):
    d_r = torch.from_numpy(r).to(dev)
    d_z = torch.full((r.size,), 123.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = f(_ints(res), _ints(bc), d_pre.data_ptr(), d_r.data_ptr(), d_z.data_ptr(),
           ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return rc, d_z.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("res,bc", [((24, 32, 24), (1, 1, 1, 1, 1, 1)),
                                    ((40, 30, 20), (1, 1, 1, 1, 0, 0))])
def test_noalloc_matches_allocating_apply_twice(res, bc):
    torch = pytest.importorskip("torch")
    p = _abi.default_params(res=res, bc=bc)
    h = Plume(p)
    precon = h.mic_diagonal()
    f = _noalloc(h.lib)
    dev = torch.device("cuda:0")
    d_pre = torch.from_numpy(precon).to(dev)
    rng = np.random.default_rng(7)
    for call in range(2):  # two calls in a row on the same scratch
        r = rng.standard_normal(h.N)
        z_ref, _ = h.mic_apply(r)
        rc, z = _call(f, torch, dev, res, bc, d_pre, r)
        assert rc == PLUME_OK
        # the same kernels in the same FP64 operation order: bit for bit
        np.testing.assert_array_equal(z, z_ref, err_msg="call %d" % call)
    h.close()


@pytest.mark.gpu
def test_noalloc_expired_wait_gives_nan_then_recovers(monkeypatch):
    """A sweep wait that runs out (the entry-gate test hook: a device flag
    that nothing sets, polled before any copy is issued) leaves z all NaN;
    the next call clears the shared state and matches plume_mic_apply."""
    torch = pytest.importorskip("torch")
    res, bc = (24, 32, 24), (1, 1, 1, 1, 1, 1)
    h = Plume(_abi.default_params(res=res, bc=bc))
    f = _noalloc(h.lib)
    dev = torch.device("cuda:0")
    d_pre = torch.from_numpy(h.mic_diagonal()).to(dev)
    r = np.random.default_rng(9).standard_normal(h.N)
    monkeypatch.setenv("PLUME_NOALLOC_WAIT_GATE", "1000")
    rc, z = _call(f, torch, dev, res, bc, d_pre, r)
    assert rc == PLUME_OK  # the expiry is reported in the output, the call only queues work
    assert np.isnan(z).all()
    monkeypatch.delenv("PLUME_NOALLOC_WAIT_GATE")
    rc, z = _call(f, torch, dev, res, bc, d_pre, r)
    assert rc == PLUME_OK
    z_ref, _ = h.mic_apply(r)
    np.testing.assert_array_equal(z, z_ref)
    h.close()


@pytest.mark.gpu
def test_noalloc_on_a_second_device():
    """The scratch array exists once per device and the sweep kernels' launch
    attributes are set per device: a call on cuda:1 after calls on cuda:0."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("one visible GPU")
    res, bc = (24, 32, 24), (1, 1, 1, 1, 0, 0)
    p = _abi.default_params(res=res, bc=bc, device=1)
    h = Plume(p)
    f = _noalloc(h.lib)
    dev = torch.device("cuda:1")
    d_pre = torch.from_numpy(h.mic_diagonal()).to(dev)
    r = np.random.default_rng(11).standard_normal(h.N)
    with torch.cuda.device(dev):
        rc, z = _call(f, torch, dev, res, bc, d_pre, r)
    assert rc == PLUME_OK
    z_ref, _ = h.mic_apply(r)
    np.testing.assert_array_equal(z, z_ref)
    h.close()
