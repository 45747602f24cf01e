"""The reference's convergence tests on the GPU: exact function 4 (the oblique sine wave) with its source
(exactfunc.f90:CalcSource CASE(4)) on the conforming and mortar meshes of regressioncheck/checks/convtest.

- Ut with the source at t = 0.37 against the oracle (1e-12), on a conforming box and a mortar mesh; ten
  LSERK steps (stage times t + c_i dt in the source) against the oracle (1e-11); the captured time loop
  (fg_run, device-side time) equal to single steps with host times.
- convtest/h_3D_mortar: N=3, AdvVel (0.3, 0.3, 0.3), Riemann 33, mu0 1e-3, CFLscale = DFLscale = 0.9,
  tend 1, FLIPPED_001/002/004/008: L2 errors below 0.5 (analyze_L2) and the mean order of convergence
  within 15 % of N+1 for at least 80 % of the variables (analyze_Convtest_h_tolerance / _rate).
- convtest/p_3D_mortar: MORTAR_002, AdvVel (0.3, 0, 0), N = 1..10: L2 errors below 5 (analyze_L2); every
  increment of N up to 8 lowers the error of every variable, and the algebraic rate
  log(e_N / e_N+1) / log((N+1) / N), averaged over the variables, exceeds 0.6 on at least 75 % of the
  increments (this file's reading of analyze_Convtest_p_rate = 0.6, analyze_Convtest_p_percentage = 0.75).
- convtest/h_3D and p_3D (conforming periodic meshes CART_HEX_PERIODIC_001..008_3D, AdvVel (0.3, 0.3, 0.3),
  p-rate 0.8) and their parabolic_off variants (Euler: mu0 = 0; h-tolerance 0.7, L2 below 0.8): the same
  criteria.
"""
import os

import numpy as np
import pytest

from _cases import l2_error, oracle_cfg, perturb_state, product_cfg, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
CONV = dict(Riemann="roeentropyfix", Lifting="br1", kappa=1.4, R=287.058, Pr=0.72, mu0=1e-3, CFLScale=0.9, DFLScale=0.9,
            IniExactFunc=4)


def _cfg(N, adv, **kw):
    return product_cfg(**dict(dict(N=N, NodeType="gauss", SplitDG="weak", AdvVel=adv, **CONV), **kw))


@pytest.mark.parametrize("mesh", ["box", "CART_HEX_PERIODIC_MORTAR_FLIPPED_002_mesh.h5"])
def test_source_parity(mesh):
    c = _cfg(4, (0.3, 0.2, 0.1), IniFrequency=1.3, IniAmplitude=0.2)
    m = fmesh.cartesian_box((3, 3, 3), (-1,) * 3, (1,) * 3) if mesh == "box" else fmesh.read_hopr(os.path.join(HOPR, mesh))
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = perturb_state(testcases.sine_wave_state(f.elem_xgp(), 0.1, (0.3, 0.2, 0.1), 1.3, 0.2), seed=2)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.37), o.time_derivative(0.37))
    assert err <= 1e-12, err
    # stepping: the source at the stage times
    t_f = t_o = 0.25
    for _ in range(10):
        dt_f, dt_o = f.CalcTimeStep()[0], o.calc_timestep()[0]
        assert abs(dt_f / dt_o - 1.0) <= 1e-12
        t_f = f.TimeStepByLSERKW2(t_f, dt_f)
        t_o = o.timestep(t_o, dt_o)
    err = rel_err(f.U, o.get_state())
    f.close()
    assert err <= 1e-11, err


def test_captured_time_loop_matches_single_steps():
    c = _cfg(3, (0.3, 0.3, 0.3))
    m = fmesh.read_hopr(os.path.join(HOPR, "CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5"))
    f, g = Flexi(c, m), Flexi(c, m)
    U0 = testcases.sine_wave_state(f.elem_xgp(), 0.0, (0.3, 0.3, 0.3))
    f.U = U0
    g.U = U0
    t_f = f.TimeDisc(6)[0]
    t_g = 0.0
    for _ in range(6):
        t_g = g.TimeStepByLSERKW2(t_g, g.CalcTimeStep()[0])
    assert abs(t_f - t_g) <= 1e-15 * t_g
    err = rel_err(f.U, g.U)
    f.close()
    g.close()
    assert err <= 1e-13, err


def _run(name, N, adv, t_end=1.0, **kw):
    f = Flexi(_cfg(N, adv, **kw), fmesh.read_hopr(os.path.join(HOPR, name)))
    x = f.elem_xgp()
    f.U = testcases.sine_wave_state(x, 0.0, adv)
    t = 0.0
    while t < t_end - 1e-12:
        dt, err = f.CalcTimeStep()
        assert err == 0
        t = f.TimeStepByLSERKW2(t, min(dt, t_end - t))
    e = l2_error(N, orc.NT_GAUSS, x, f.mesh_array("sJ"), f.U, lambda xa: testcases.sine_wave_state(xa, t_end, adv))
    f.close()
    return e


def test_h_convergence_mortar_gpu():
    errs = np.array([_run(f"CART_HEX_PERIODIC_MORTAR_FLIPPED_{k:03d}_mesh.h5", 3, (0.3, 0.3, 0.3)) for k in (1, 2, 4, 8)])
    assert (errs < 0.5).all()
    order = np.log2(errs[:-1] / errs[1:]).mean(axis=0)
    ok = np.abs(order / 4.0 - 1.0) <= 0.15
    assert ok.mean() >= 0.8, order
    # the oracle's errors on FLIPPED_001 (same discretisation, oracle run of tests/test_oracle_mortar.py's setting)
    assert np.allclose(errs[0], [0.08069912, 0.07014683, 0.0655366, 0.08004052, 0.1400404], rtol=1e-6)


def test_p_convergence_mortar_gpu():
    errs = np.array([_run("CART_HEX_PERIODIC_MORTAR_002_mesh.h5", N, (0.3, 0.0, 0.0)) for N in range(1, 11)])
    assert (errs < 5.0).all()
    assert (errs[1:8] < errs[:7]).all(), errs
    rate = np.log(errs[:-1] / errs[1:]) / np.log(np.arange(2, 11) / np.arange(1, 10))[:, None]
    assert (rate.mean(axis=1) > 0.6).mean() >= 0.75, rate


@pytest.mark.parametrize("mu0,tol,l2max", [(1e-3, 0.15, 0.5), (0.0, 0.7, 0.8)])
def test_h_convergence_conforming_gpu(mu0, tol, l2max):
    errs = np.array([_run(f"CART_HEX_PERIODIC_{k:03d}_3D_mesh.h5", 3, (0.3, 0.3, 0.3), mu0=mu0) for k in (1, 2, 4, 8)])
    assert (errs < l2max).all()
    order = np.log2(errs[:-1] / errs[1:]).mean(axis=0)
    assert (np.abs(order / 4.0 - 1.0) <= tol).mean() >= 0.8, order


@pytest.mark.parametrize("mu0", [1e-3, 0.0])
def test_p_convergence_conforming_gpu(mu0):
    errs = np.array([_run("CART_HEX_PERIODIC_002_3D_mesh.h5", N, (0.3, 0.3, 0.3), mu0=mu0) for N in range(1, 11)])
    assert (errs < 5.0).all()
    rate = np.log(errs[:-1] / errs[1:]) / np.log(np.arange(2, 11) / np.arange(1, 10))[:, None]
    assert (rate.mean(axis=1) > 0.8).mean() >= 0.75, rate
