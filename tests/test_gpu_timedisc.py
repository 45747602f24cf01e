"""The time loop of fg_run against the restated control logic of FLEXI's TimeDisc (oracle/timedisc.py driving the
CPU oracle): UpdateTimeStep's clipping to the analysis times and to TEnd with the dt/100 stretch, the
nCalcTimeStepMax reuse of the time step, dtmin and the dtkill abort of EvalTimeStep, maxIter, and the NaN-density
abort of CALCTIMESTEP (timedisc_func.f90:215-268,433-454, timedisc.f90:190-212, calctimestep.f90:157-160).
Failures are made on the host (a time-step bound above the CFL time step, a NaN written into the host state);
nothing faults or hangs the GPU."""
import math

import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, FlexiError, make_config
from oracle import oracle as orc
from oracle.timedisc import KillTimestep, TimeDiscLoop

pytestmark = pytest.mark.gpu

FG_ERR_NAN, FG_ERR_DTKILL = 5, 7
STATE_TOL = 1e-10
BASE = dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1", kappa=1.4, R=71.42857, Pr=0.72, mu0=1.0 / 1600.0,
            CFLScale=0.9, DFLScale=0.9)


def pair(meshes=None, **kw):
    c = make_config(**dict(BASE, **kw))
    m = meshes or fmesh.tgv_box(3, ngeo=2, perturb=0.1, seed=2)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.1, kappa=c.kappa, R=c.R), seed=5)
    f.U = U0
    o.set_state(U0)
    return f, o, U0


def loop_for(o, **kw):
    return TimeDiscLoop(o.calc_timestep, o.timestep, **kw)


def run_gpu_to_end(f, chunk=1000, max_calls=100):
    """fg_run until the instance finished; returns the times at which it held on an analysis time."""
    held = []
    for _ in range(max_calls):
        f.TimeDisc(chunk)
        st = f.timedisc_state()[0]
        if st["finished"]:
            return held, st
        assert st["atAnalyze"], st
        held.append(st["t"])
    raise AssertionError("no end time reached")


def test_tend_and_analysis_times():
    tEnd, adt = 0.2, 0.07
    f, o, _ = pair(TEnd=tEnd, Analyze_dt=adt)
    held, st = run_gpu_to_end(f)
    lp = loop_for(o, tEnd=tEnd, analyze_dt=adt)
    lp.run(10000)
    assert lp.doFinalize
    # every analysis time and the end are hit (up to the round-off of t + (tAnalyze - t))
    assert np.allclose(held, lp.analyze_times[:-1], rtol=1e-13, atol=0) and len(held) == 2, (held, lp.analyze_times)
    assert abs(held[0] - adt) <= 1e-15 and abs(held[1] - 2 * adt) <= 1e-15
    assert st["t"] == pytest.approx(tEnd, rel=1e-15, abs=0) and st["iter"] == lp.iter
    Uend = f.U
    e = rel_err(Uend, o.get_state())
    # a finished instance does not advance
    f.TimeDisc(5)
    st2 = f.timedisc_state()[0]
    assert st2["t"] == st["t"] and st2["iter"] == st["iter"] and np.array_equal(f.U, Uend)
    f.close()
    assert e <= STATE_TOL, e


def test_stretch_to_end_time():
    """A final step that would leave less than dt/100 to TEnd is stretched to TEnd (timedisc_func.f90:266)."""
    f0, o0, U0 = pair()
    dt0, _ = f0.CalcTimeStep()
    f0.close()
    tEnd = 3.005 * dt0  # after three CFL steps 0.005 dt remains: the third step is stretched to TEnd
    f, o, _ = pair(TEnd=tEnd)
    held, st = run_gpu_to_end(f)
    lp = loop_for(o, tEnd=tEnd)
    lp.run(100)
    assert held == [] and st["iter"] == lp.iter and st["t"] == tEnd and lp.t == tEnd
    e = rel_err(f.U, o.get_state())
    f.close()
    assert e <= STATE_TOL, e


def test_ncalctimestepmax_reuse():
    f, o, _ = pair(nCalcTimeStepMax=5)
    f.TimeDisc(40)
    st = f.timedisc_state()[0]
    lp = loop_for(o, nCalcTimeStepMax=5)
    lp.run(40)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert st["iter"] == 40 and abs(st["t"] - lp.t) <= 1e-12 * lp.t and e <= STATE_TOL, (st, lp.t, e)


def test_dtmin_limits_the_step():
    f0, _, _ = pair()
    dt0, _ = f0.CalcTimeStep()
    f0.close()
    dtmin = 1.5 * dt0
    f, o, _ = pair(dtmin=dtmin, CFLScale=0.3, DFLScale=0.3)
    dtc, _ = f.CalcTimeStep()
    assert dtc < dtmin
    f.TimeDisc(6)
    st = f.timedisc_state()[0]
    lp = loop_for(o, dtmin=dtmin)
    lp.run(6)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert st["nDtLimited"] == lp.nDtLimited == 6 and st["dt"] == dtmin and st["t"] == pytest.approx(6 * dtmin, rel=1e-14)
    assert e <= STATE_TOL, e


def test_dtkill_stops_the_run():
    f, o, U0 = pair()
    dt0, _ = f.CalcTimeStep()
    f.close()
    f, o, U0 = pair(dtkill=2.0 * dt0)
    with pytest.raises(FlexiError) as ex:
        f.TimeDisc(3)
    assert ex.value.code == FG_ERR_DTKILL
    # the state where the critical time step was found is kept
    assert np.array_equal(f.U, U0)
    st = f.timedisc_state()[0]
    assert st["iter"] == 0 and st["t"] == 0.0
    f.close()
    with pytest.raises(KillTimestep):
        loop_for(o, dtkill=2.0 * dt0).run(3)


def test_nan_density_stops_the_run():
    f, o, U0 = pair()
    U = U0.copy()
    U[1, 2, 1, 0, 0] = np.nan  # density of one node, written into the host state
    f.U = U
    with pytest.raises(FlexiError) as ex:
        f.TimeDisc(2)
    assert ex.value.code == FG_ERR_NAN
    f.close()


def test_maxiter():
    f, o, _ = pair(maxIter=7)
    f.TimeDisc(20)
    st = f.timedisc_state()[0]
    lp = loop_for(o, maxIter=7)
    lp.run(20)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert st["finished"] and st["iter"] == 7 == lp.iter and abs(st["t"] - lp.t) <= 1e-12 * lp.t and e <= STATE_TOL


def test_set_time_restarts_the_loop():
    tEnd = 0.1
    f, o, U0 = pair(TEnd=tEnd)
    run_gpu_to_end(f)
    f.U = U0
    f.set_time(0.0)
    st = f.timedisc_state()[0]
    assert st["iter"] == 0 and not st["finished"] and st["t"] == 0.0
    held, st = run_gpu_to_end(f)
    lp = loop_for(o, tEnd=tEnd)
    lp.run(1000)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert st["t"] == tEnd and st["iter"] == lp.iter and e <= STATE_TOL


def test_ensemble_instances_end_independently():
    """Two instances of different Mach number reach TEnd after different step counts; each equals its own run."""
    c = make_config(**dict(BASE, TEnd=0.1, Analyze_dt=0.04))
    meshes = [fmesh.tgv_box(2), fmesh.tgv_box(3)]
    machs = [0.1, 0.3]
    ens = fmesh.concatenate(meshes)
    f = Flexi(c, ens)
    x = f.elem_xgp()
    U0 = np.concatenate([perturb_state(testcases.tgv_state(x[ens.elem_inst == i], mach=machs[i], kappa=c.kappa, R=c.R), seed=i)
                         for i in range(2)])
    f.U = U0
    for _ in range(50):
        f.TimeDisc(1000)
        if all(s["finished"] for s in f.timedisc_state()):
            break
    sts = f.timedisc_state()
    Uf = f.U
    f.close()
    off = 0
    iters = []
    for i, m in enumerate(meshes):
        o = orc.Oracle(oracle_cfg(c), m)
        o.set_state(U0[off:off + m.n_elems])
        lp = loop_for(o, tEnd=0.1, analyze_dt=0.04)
        lp.run(10000)
        assert sts[i]["finished"] and sts[i]["iter"] == lp.iter and sts[i]["t"] == pytest.approx(0.1, rel=1e-15)
        assert rel_err(Uf[off:off + m.n_elems], o.get_state()) <= STATE_TOL
        iters.append(lp.iter)
        off += m.n_elems
    assert iters[0] != iters[1]
