"""Many independent plumes on one GPU (include/plume_batch.h).

 * the batched-plume randomisation;
 * the fused engine's host-side checks (CPU: unsupported parameter
   combinations are refused before any device work);
 * fused engine, FP64: every plume of an uneven batch equals the FP64 oracle
   of its own configuration (FLUID_3D_MIC::step, FLUID_3D_MIC.cpp:179-223)
   within 1e-9 relative L2 and +-1 iteration, as the single-plume FP64 engine
   does;
 * fused engine, FP32: plumes of the batched configuration itself (grids up
   to 96x128x96) against the same plumes stepped alone by the single-plume
   FP32 engine, within the FP32 configuration's 1e-4 bound;
 * the step graph and the host-driven loop give identical bits;
 * the autotuner writes its choices to the JSON cache and a second batch of
   the same shape reads them back;
 * streams engine: stepping instances concurrently gives each instance
   exactly the fields it gets when stepped alone.
"""
import json
import os

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from cfs_plume_gb300.batch import PlumeBatch, batch_params
from cfs_plume_gb300.plume import PlumeError

GRIDS = {(32, 32, 32), (48, 64, 48), (64, 96, 64), (96, 128, 96)}


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


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


@pytest.mark.parametrize("bad", [
    dict(source=_abi.SRC_COLUMN),
    dict(warm_start=_abi.WARM_LEARNED),
    dict(preconditioner=_abi.PRECOND_NET),
    dict(res=(300, 20, 20)),
])
def test_fused_batch_refuses_unsupported_plumes(bad):
    """Checked on the host before any device call (runs without a GPU)."""
    good = _abi.plume_config((16, 20, 12))
    bad_p = _abi.plume_config(bad.pop("res", (16, 20, 12)), **bad)
    with pytest.raises(PlumeError) as e:
        PlumeBatch([good, bad_p])
    assert e.value.status == 7  # PLUME_ERR_UNSUPPORTED
    assert "plume 1" in str(e.value)


def test_fused_batch_refuses_mixed_precision():
    a = _abi.plume_config((16, 20, 12), precision=_abi.PREC_FP32)
    b = _abi.plume_config((16, 20, 12), precision=_abi.PREC_FP64)
    with pytest.raises(PlumeError) as e:
        PlumeBatch([a, b])
    assert e.value.status == 7


# uneven plumes with every boundary and solver variant the fused engine takes
UNEVEN = [
    dict(res=(16, 20, 12), bc=(1, 1, 1, 1, 1, 1), vorticity_eps=2.0, buoyancy=1.0,
         box_lo=(6, 1, 4), box_hi=(10, 4, 8), seed=3),
    dict(res=(17, 23, 13), bc=(1, 1, 1, 1, 1, 1), vorticity_eps=1.0, buoyancy=1.0,
         box_lo=(6, 2, 4), box_hi=(11, 6, 9), seed=7, warm_start=_abi.WARM_PREVIOUS),
    dict(res=(20, 16, 18), bc=(0, 0, 0, 0, 0, 0), vorticity_eps=1.5, buoyancy=0.5,
         box_lo=(7, 1, 7), box_hi=(13, 4, 11), seed=11),
    dict(res=(24, 32, 24), bc=(0, 1, 0, 1, 0, 1), vorticity_eps=0.0, buoyancy=2.0,
         box_lo=(9, 1, 9), box_hi=(15, 4, 15), seed=13, criterion=_abi.CRIT_REFERENCE, tol=1e-10),
    dict(res=(40, 12, 10), bc=(1, 1, 1, 1, 1, 1), vorticity_eps=3.0, buoyancy=1.0,
         box_lo=(15, 1, 3), box_hi=(25, 3, 7), seed=17, warm_start=_abi.WARM_PREVIOUS),
]


def uneven(precision, tol=1e-10):
    out = []
    for kw in UNEVEN:
        kw = dict(kw)
        kw.setdefault("criterion", _abi.CRIT_REL2)
        kw.setdefault("tol", tol)
        res = kw.pop("res")
        out.append(_abi.plume_config(res, precision=precision, **kw))
    return out


@pytest.mark.gpu
def test_fused_batch_fp64_matches_the_oracle_per_plume():
    from oracle import oracle
    params = uneven(_abi.PREC_FP64)
    b = PlumeBatch(params, tune=False)
    steps = 4
    _, stats = b.run(0, steps)
    for i, p in enumerate(params):
        o = oracle.Oracle(p)
        oi = []
        for s in range(steps):
            o.add_source(s)
            oi.append(o.step().iterations)
        gi = [st.iterations for st in stats[i]]
        assert all(abs(a - c) <= 1 for a, c in zip(gi, oi)), (i, gi, oi)
        for name in ("velocity", "density", "heat", "pressure"):
            e = rel_l2(b.field(i, name), o.field(name))
            assert e < 1e-9, (i, name, e)
        o.close()
    b.close()


@pytest.mark.gpu
def test_fused_batch_fp32_configuration_plumes_match_single_plumes():
    """Eight plumes of the batched configuration (seed 5: every grid size up
    to 96x128x96), 10 steps, FP32 fields at rel-L2 1e-6: each within 1e-4
    relative L2 of the same plume stepped alone, every solve converged."""
    from cfs_plume_gb300.plume import Plume
    params = [batch_params(5, i) for i in range(8)]
    assert {tuple(p.res) for p in params} == GRIDS
    b = PlumeBatch(params)
    steps = 10
    _, stats = b.run(0, steps)
    for i, p in enumerate(params):
        assert all(s.converged == 1 and s.rel_residual <= 1e-6 for s in stats[i]), i
        h = Plume(p)
        alone = []
        for s in range(steps):
            h.add_source(s)
            alone.append(h.step().iterations)
        for name in ("velocity", "density"):
            e = rel_l2(b.field(i, name), h.field(name))
            assert e < 1e-4, (i, tuple(p.res), name, e)
        gi = [s.iterations for s in stats[i]]
        assert all(abs(a - c) <= max(2, c // 20) for a, c in zip(gi, alone)), (i, gi, alone)
        h.close()
    b.close()


@pytest.mark.gpu
def test_fused_batch_fp32_configuration_plumes_against_fp64_oracle():
    """Plumes of the batched configuration itself (seed 5's 32^3 and 48x64x48
    instances), FP32 fields with FP64-class reductions at rel-L2 1e-6, 20
    steps in one fused batch: each within 1e-4 relative L2 of the FP64 oracle
    of its own configuration (FLUID_3D_MIC::step at the same stop test),
    inside the plume's predictability horizon."""
    from oracle import oracle
    cand = [batch_params(5, i) for i in range(16)]
    params = [p for p in cand if tuple(p.res) == (32, 32, 32)][:2] + \
             [p for p in cand if tuple(p.res) == (48, 64, 48)][:2]
    assert len(params) == 4
    b = PlumeBatch(params)
    steps = 20
    _, stats = b.run(0, steps)
    for i, p in enumerate(params):
        q = _abi.PlumeParams.from_buffer_copy(bytes(p))
        q.precision = _abi.PREC_FP64
        o = oracle.Oracle(q)
        for s in range(steps):
            o.add_source(s)
            o.step()
        assert all(st.converged == 1 and st.rel_residual <= 1e-6 for st in stats[i]), i
        for name in ("velocity", "density"):
            e = rel_l2(b.field(i, name), o.field(name))
            assert e < 1e-4, (i, tuple(p.res), name, e)
        o.close()
    b.close()


@pytest.mark.gpu
def test_batched_configuration_runs_its_100_steps():
    """The batched configuration as specified: 64 plumes of uneven grids, 100
    steps each in one fused batch; every solve meets its stop test and every
    field stays finite."""
    params = [batch_params(11, i) for i in range(64)]
    b = PlumeBatch(params)
    _, stats = b.run(0, 100)
    bad = [(i, k) for i in range(64) for k, st in enumerate(stats[i])
           if not (st.converged == 1 and st.rel_residual <= 1e-6)]
    assert not bad, bad[:5]
    for i in (0, 21, 42, 63):
        for name in ("velocity", "density", "pressure"):
            assert np.isfinite(b.field(i, name)).all(), (i, name)
    b.close()


@pytest.mark.gpu
def test_fused_graph_and_host_loop_are_identical():
    params = uneven(_abi.PREC_FP32, tol=1e-6)
    a = PlumeBatch(params, graph=True, tune=False)
    c = PlumeBatch(params, graph=False, tune=False)
    assert a.tuning()["graph"] is True and c.tuning()["graph"] is False
    _, sa = a.run(0, 3)
    _, sc = c.run(0, 3)
    for i in range(len(params)):
        assert [s.iterations for s in sa[i]] == [s.iterations for s in sc[i]]
        for name in ("velocity", "density", "pressure"):
            assert np.array_equal(a.field(i, name), c.field(i, name)), (i, name)
    a.close()
    c.close()


@pytest.mark.gpu
def test_cg_groups_change_no_bit():
    """Ten plumes of the configuration (every grid size) as one CG group and as
    two groups advanced in parallel graph branches with persistent stage
    launches: each plume's arithmetic depends neither on its group nor on the
    grid walking its virtual blocks, so the fields are identical bit for bit;
    and the two-group graph equals its host-driven loop."""
    params = [batch_params(5, i) for i in range(10)]
    one = PlumeBatch(params, groups=1, tune=False)
    two = PlumeBatch(params, groups=2, tune=False, persistent=True)
    two_host = PlumeBatch(params, groups=2, tune=False, graph=False)
    assert one.tuning()["groups"] == 1 and two.tuning()["groups"] == 2
    assert {c["group"] for c in two.tuning()["classes"]} == {0, 1}
    runs = [b.run(0, 3)[1] for b in (one, two, two_host)]
    for i in range(len(params)):
        its = [[s.iterations for s in r[i]] for r in runs]
        assert its[0] == its[1] == its[2], (i, its)
        for name in ("velocity", "density", "pressure"):
            a = one.field(i, name)
            assert np.array_equal(a, two.field(i, name)), (i, name)
            assert np.array_equal(a, two_host.field(i, name)), (i, name)
    for b in (one, two, two_host):
        b.close()


@pytest.mark.gpu
def test_autotuner_writes_and_reads_its_cache(tmp_path):
    cache = str(tmp_path / "tune" / "cache.json")
    params = [batch_params(9, i) for i in range(6)]
    a = PlumeBatch(params, tune_cache=cache)
    ta = a.tuning()
    assert ta["timed"] is True and ta["from_cache"] is False and ta["cache_written"] is True
    with open(cache) as f:
        entries = json.load(f)
    assert ta["signature"] in entries
    e = entries[ta["signature"]]
    assert e["cells_epb"] == ta["cells_epb"] and e["bz"] == [c["bz"] for c in ta["classes"]]
    assert e["pf"] == [c["pf"] for c in ta["classes"]]
    for c in ta["classes"]:
        assert [c["bz"], c["pf"]] in [sh[:2] for sh in c["shape_candidates"]] and c["slabs"] <= 16
    a.run(0, 2)
    a.close()
    b = PlumeBatch(params, tune_cache=cache)
    tb = b.tuning()
    assert tb["from_cache"] is True and tb["timed"] is False
    assert [(c["bz"], c["pf"]) for c in tb["classes"]] == [(c["bz"], c["pf"]) for c in ta["classes"]]
    b.run(0, 2)
    b.close()


@pytest.mark.gpu
def test_fused_batch_has_no_handles():
    b = PlumeBatch(uneven(_abi.PREC_FP32, tol=1e-6)[:2], tune=False)
    with pytest.raises(PlumeError) as e:
        b.handle(0)
    assert e.value.status == 8  # PLUME_ERR_STATE
    b.close()


def _small(seed, i, res):
    p = batch_params(seed, i)
    q = _abi.plume_config(res, seed=p.seed, buoyancy=p.buoyancy, vorticity_eps=p.vorticity_eps)
    return q


@pytest.mark.gpu
def test_concurrent_instances_match_instances_stepped_alone():
    from cfs_plume_gb300.plume import Plume
    params = [_small(3, 0, (24, 32, 24)), _small(3, 1, (32, 48, 32)), _small(3, 2, (16, 24, 16))]
    b = PlumeBatch(params, engine="streams")
    secs, stats = b.run(0, 4, threads=0)
    assert secs > 0 and all(len(s) == 4 for s in stats)
    for i, p in enumerate(params):
        h = Plume(p)
        alone = []
        for s in range(4):
            h.add_source(s)
            alone.append(h.step())
        ref = h.field("velocity")
        h.close()
        b.handle(i)  # the streams engine keeps a handle per instance
        np.testing.assert_array_equal(b.field(i, "velocity"), ref)
        assert [s.iterations for s in stats[i]] == [s.iterations for s in alone]
    b.close()
