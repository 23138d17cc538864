"""Many independent plumes on one GPU (include/plume_batch.h): the
batched-plume randomisation, and that stepping instances concurrently gives
each instance exactly the fields it gets when stepped alone."""
import ctypes as C

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from cfs_plume_gb300.batch import PlumeBatch, batch_params

GRIDS = {(32, 32, 32), (48, 64, 48), (64, 96, 64), (96, 128, 96)}


def test_batch_params_follow_the_configuration():
    seen = set()
    for i in range(64):
        p = batch_params(7, i)
        res = tuple(p.res)
        seen.add(res)
        assert res in GRIDS
        assert tuple(p.bc) == (1,) * 6
        assert 0.5 <= p.buoyancy <= 2.0 and 0.0 <= p.vorticity_eps <= 4.0
        assert p.precision == _abi.PREC_FP32 and p.criterion == _abi.CRIT_REL2 and p.tol == 1e-6
        assert p.source == _abi.SRC_BOX and p.source_noise == 0.05 and p.seed == 7 + i
        X, Y, Z = res
        for k, n in ((0, X), (2, Z)):  # box centre in the middle third of the floor
            c = 0.5 * (p.box_lo[k] + p.box_hi[k])
            assert n / 3.0 - 1.0 <= c <= 2.0 * n / 3.0 + 1.0
            assert 1 <= p.box_lo[k] < p.box_hi[k] <= n - 1
        assert p.box_lo[1] == 2 * Y // 64 and p.box_hi[1] == 6 * Y // 64
        q = batch_params(7, i)  # deterministic
        assert bytes(p) == bytes(q)
    assert seen == GRIDS


def _small(seed, i, res):
    p = batch_params(seed, i)
    q = _abi.plume_config(res, seed=p.seed, buoyancy=p.buoyancy, vorticity_eps=p.vorticity_eps)
    return q


@pytest.mark.gpu
def test_concurrent_instances_match_instances_stepped_alone():
    from cfs_plume_gb300.plume import Plume
    params = [_small(3, 0, (24, 32, 24)), _small(3, 1, (32, 48, 32)), _small(3, 2, (16, 24, 16))]
    b = PlumeBatch(params)
    secs, stats = b.run(0, 4, threads=0)
    assert secs > 0 and all(len(s) == 4 for s in stats)
    lib = b.lib
    for i, p in enumerate(params):
        h = Plume(p)
        alone = []
        for s in range(4):
            h.add_source(s)
            alone.append(h.step())
        ref = h.field("velocity")
        h.close()
        got = np.empty(3 * p.res[0] * p.res[1] * p.res[2])
        rc = lib.plume_download(b.handle(i), _abi.FIELD_ID["velocity"], got.ctypes.data, got.size)
        assert rc == 0
        np.testing.assert_array_equal(got, ref)
        assert [s.iterations for s in stats[i]] == [s.iterations for s in alone]
    b.close()
