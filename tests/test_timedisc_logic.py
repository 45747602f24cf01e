"""CPU checks of the restated TimeDisc control (oracle/timedisc.py), the checker of fg_run's device-side
UpdateTimeStep, on synthetic time-step sequences, and of the new parameter-file keys."""
import math

import pytest

from oracle.timedisc import KillTimestep, TimeDiscLoop


def make_loop(dts, **kw):
    it = iter(dts)
    seen = []
    lp = TimeDiscLoop(lambda: (next(it), 0), lambda t, dt: seen.append((t, dt)), **kw)
    return lp, seen


def test_analysis_and_end_clipping():
    lp, seen = make_loop([0.3] * 20, tEnd=1.0, analyze_dt=0.5)
    lp.run(20)
    # 0.3, then clipped to the analysis time 0.5, 0.3, clipped to 1.0
    assert [round(dt, 12) for _, dt in seen] == [0.3, 0.2, 0.3, 0.2]
    assert lp.analyze_times == pytest.approx([0.5, 1.0]) and lp.doFinalize and lp.t == pytest.approx(1.0)


def test_stretch_rule():
    # 1.0 - 3 * 0.33 = 0.01 < 0.33/100 is false; 1.0 - 3 * 0.333 = 0.001 < 0.00333: third step stretched to the end
    lp, seen = make_loop([0.333] * 10, tEnd=1.0)
    lp.run(10)
    assert len(seen) == 3 and lp.t == 1.0 and seen[-1][1] == pytest.approx(1.0 - 2 * 0.333)


def test_analyze_dt_zero_means_tend():
    lp, _ = make_loop([0.25] * 10, tEnd=1.0, analyze_dt=0.0)
    lp.run(10)
    assert lp.analyze_times == [1.0]


def test_ncalctimestep_counts():
    # constant dt: after the first update |dt_old/dt - 1| = 0 -> floor(|log10(eps)|) = 15 -> min(15, max) - 1 skips
    calls = []

    def calc():
        calls.append(1)
        return 0.1, 0

    lp = TimeDiscLoop(calc, lambda t, dt: None, nCalcTimeStepMax=4)
    lp.run(13)
    # first update: dt_minOld = -999 -> log10(~1e8) -> 8 -> min(8,4)-1 = 3 skips; then 3 skips after every update
    assert len(calls) == 4 and lp.iter == 13
    q = abs(-999.0 / 0.1 - 1.0) ** 2 * 100.0
    assert math.floor(abs(math.log10(q))) >= 4


def test_dtmin_and_dtkill():
    lp, seen = make_loop([0.01, 0.5, 0.01], dtmin=0.1)
    lp.run(3)
    assert [dt for _, dt in seen] == [0.1, 0.5, 0.1] and lp.nDtLimited == 2
    lp, _ = make_loop([0.5, 0.01], dtkill=0.1)
    with pytest.raises(KillTimestep):
        lp.run(3)
    assert lp.iter == 1


def test_maxiter():
    lp, _ = make_loop([0.1] * 10, maxIter=4)
    lp.run(10)
    assert lp.iter == 4 and lp.doFinalize and lp.analyze_times == [pytest.approx(0.4)]


def test_ini_keys():
    from flexi_gb300.solver import config_from_ini, make_config
    c = config_from_ini("tEnd = 13.\nAnalyze_dt = 0.5 ! comment\ndtmin = 1e-9\ndtkill=1e-12\nnCalcTimeStepMax = 3\nmaxIter = 100\n")
    assert (c.TEnd, c.Analyze_dt, c.dtmin, c.dtkill, c.nCalcTimeStepMax, c.maxIter) == (13.0, 0.5, 1e-9, 1e-12, 3, 100)
    d = make_config()
    assert math.isinf(d.TEnd) and d.Analyze_dt == 0.0 and d.dtmin == -1.0 and d.dtkill == -1.0 and d.nCalcTimeStepMax == 1 and d.maxIter == -1
