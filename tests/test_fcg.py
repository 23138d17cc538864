"""Flexible CG with the network as the preconditioner stage
(PLUME_PRECOND_NET): the engine's FCG(1) loop against its CPU restatement
(oracle/fcg_oracle.py), which follows the reference's PCG loop
(FLUID_3D_MIC.cpp:951-1013) with z = net(r) in place of
applyMICPreconditioner.

The oracle is pinned two ways: with MIC(0) as M it takes exactly the
iterations of the oracle's MIC-PCG (itself bit-exact against the compiled
reference), and the fixture tests/golden/oracle_fcg_48x64x48.npz
(make_golden_fcg.py) records its network-preconditioned run.
"""
import os

import numpy as np
import pytest

from cfs_plume_gb300 import _abi
from oracle import fcg_oracle as fo
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
WEIGHTS = os.path.join(ROOT, "cfs_plume_gb300", "weights", "unet_warmstart.bin")


def plume_rhs(res, steps):
    p = _abi.plume_config(res, precision=_abi.PREC_FP64)
    o = oracle.Oracle(p)
    for s in range(steps):
        o.add_source(s)
        o.step()
    return p, o.field("divergence")


def centred(x, res):
    m = fo.interior(res)
    v = x[m]
    return v - v.mean()


def test_fcg_with_mic_takes_the_pcg_iterations():
    """With a fixed SPD preconditioner (MIC(0)) FCG is PCG: the same
    iteration count as the oracle's MIC-PCG at the same rel-L2 stop test."""
    res = (24, 32, 24)
    p, b = plume_rhs(res, 6)
    bc = tuple(p.bc)
    _, it, hist = fo.fcg(res, bc, b, fo.MicPreconditioner(res, bc), tol=1e-6)
    _, st = oracle.solve_poisson(_abi.plume_config(res, precision=_abi.PREC_FP64), b)
    assert it == st.iterations and hist[-1] <= 1e-6


def test_fixture_pins_the_oracle():
    """The fixture's MIC(0) run recomputed here gives the same count; the
    network-preconditioned count it stores is the one the GPU test checks."""
    f = np.load(os.path.join(GOLDEN, "oracle_fcg_48x64x48.npz"))
    res = tuple(int(v) for v in f["res"])
    p, b = plume_rhs(res, int(f["steps"]))
    assert np.linalg.norm(b) == pytest.approx(float(f["b_l2"]), rel=1e-12)
    bc = tuple(p.bc)
    _, it, _ = fo.fcg(res, bc, b, fo.MicPreconditioner(res, bc), tol=float(f["tol"]))
    assert it == int(f["iters_mic"])
    assert int(f["iters_net"]) < int(f["iters_mic"])
    assert f["hist_net"][-1] <= float(f["tol"])


def test_network_file_reader():
    params, kind, c = fo.load_net_file(WEIGHTS)
    assert params.size == fo.uo.num_params() and kind in (0, 1) and c > 0


@pytest.mark.gpu
def test_gpu_fcg_network_matches_oracle():
    """FP64 handle, network preconditioner: the GPU FCG solve of the fixture's
    right-hand side takes the oracle's iteration count within one (the
    network runs in BF16 with FP32 accumulation on the GPU, float64
    accumulation in the oracle), meets the stop test, and its solution
    agrees with the oracle's up to the closed box's constant."""
    from cfs_plume_gb300.net import PlumeNet
    from cfs_plume_gb300.plume import Plume
    f = np.load(os.path.join(GOLDEN, "oracle_fcg_48x64x48.npz"))
    res = tuple(int(v) for v in f["res"])
    p, b = plume_rhs(res, int(f["steps"]))
    g = Plume(_abi.plume_config(res, precision=_abi.PREC_FP64, preconditioner=_abi.PRECOND_NET))
    net = PlumeNet(path=WEIGHTS)
    net.attach(g)
    x, st = g.solve_poisson(b)
    assert abs(st.iterations - int(f["iters_net"])) <= 1, (st.iterations, int(f["iters_net"]))
    assert st.converged == 1 and st.rel_residual <= float(f["tol"])
    # the true residual of the returned solution
    r = np.where(fo.interior(res), b - oracle.mult_a(res, tuple(p.bc), x), 0.0)
    assert np.linalg.norm(r) <= 1.5 * float(f["tol"]) * np.linalg.norm(b)
    stride = int(f["stride"])
    xo = np.zeros_like(b)
    xo[::stride] = f["x_net"]
    sel = np.zeros(b.size, dtype=bool)
    sel[::stride] = True
    m = fo.interior(res) & sel
    a, o = x[m] - x[m].mean(), xo[m] - xo[m].mean()
    assert np.linalg.norm(a - o) / np.linalg.norm(o) < 1e-4
    g.close()
    net.close()


@pytest.mark.gpu
def test_gpu_fcg_plume_steps_converge_like_plain():
    """FP32 plume steps solved by network-preconditioned FCG: every solve meets
    the rel-L2 1e-6 test without falling back, in fewer iterations than
    MIC-PCG, and the velocity stays within 1e-4 relative L2 of the plain
    MIC-PCG arm's."""
    from cfs_plume_gb300.net import PlumeNet
    from cfs_plume_gb300.plume import Plume
    res = (48, 64, 48)
    plain = Plume(_abi.plume_config(res))
    flex = Plume(_abi.plume_config(res, preconditioner=_abi.PRECOND_NET))
    net = PlumeNet(path=WEIGHTS)
    net.attach(flex)
    ip, ifl = [], []
    for s in range(8):
        for h in (plain, flex):
            h.add_source(s)
        ip.append(plain.step().iterations)
        st = flex.step()
        ifl.append(st.iterations)
        assert st.converged == 1 and st.fallback == 0 and st.rel_residual <= 1e-6, s
    assert np.mean(ifl[2:]) < 0.75 * np.mean(ip[2:]), (ifl, ip)
    vp, vf = plain.field("velocity"), flex.field("velocity")
    assert np.linalg.norm(vf - vp) / np.linalg.norm(vp) < 1e-4
    plain.close()
    flex.close()
    net.close()
