"""Overintegration on the GPU (overintegration.f90, dg.f90:663-675, timedisc.f90:115-123) against the oracle.

Bars as in test_gpu_parity.py: Ut after one right-hand side within 1e-12 and the state after LSERK steps
within 1e-10 (max abs error per variable / that variable's max); the state filter within 1e-13; the
CALCTIMESTEP time step (CFL on MIN(N, NUnder), the Gauss table for Gauss-Lobatto nodes) within 1e-13.
The conservative cut-off's 1/J on NUnder is formed from the projection of 1/sJ here and from DetJac_Ref
in the oracle, as the reference does: the two agree to round-off.
"""
import numpy as np
import pytest

from _cases import channel_pair, product_cfg, rel_err, tgv_pair

pytestmark = pytest.mark.gpu

CASES = {
    "gauss5_weak_cutoff3": dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", OverintegrationType=1, NUnder=3),
    "gauss5_weak_conscutoff3": dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roe", OverintegrationType=2, NUnder=3),
    "gl7_split_pi_cutoff5_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2",
                                     OverintegrationType=1, NUnder=5),
    "gl4_weak_conscutoff2": dict(N=4, NodeType="gauss-lobatto", SplitDG="weak", Riemann="lf", OverintegrationType=2, NUnder=2),
    "gauss11_weak_cutoff7": dict(N=11, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", OverintegrationType=1, NUnder=7),
    "gauss3_split_pi_conscutoff2": dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", OverintegrationType=2,
                                        NUnder=2),
}
COMMON = dict(kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.9, DFLScale=0.9)


@pytest.mark.parametrize("name", list(CASES))
def test_rhs_parity(name):
    c = product_cfg(**CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3, ngeo=2, perturb=0.1, seed=4)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


@pytest.mark.parametrize("name", ["gauss5_weak_cutoff3", "gauss5_weak_conscutoff3", "gl4_weak_conscutoff2"])
def test_state_filter_and_dt(name):
    c = product_cfg(**CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3, ngeo=2, perturb=0.1, seed=5)
    f.overintegrate_state()
    o.overintegrate_state()
    assert rel_err(f.U, o.get_state()) <= 1e-13
    dtf, errf = f.CalcTimeStep()
    dto, erro = o.calc_timestep()
    f.close()
    assert errf == 0 and erro == 0 and abs(float(np.atleast_1d(dtf)[0]) - dto) <= 1e-13 * dto


@pytest.mark.parametrize("name", ["gauss5_weak_cutoff3", "gauss5_weak_conscutoff3", "gl7_split_pi_cutoff5_br2"])
def test_lserk_steps(name):
    c = product_cfg(**CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3, ngeo=2, perturb=0.1, seed=6)
    f.overintegrate_state()
    o.overintegrate_state()
    tf = to = 0.0
    for _ in range(10):
        dt, err = o.calc_timestep()
        assert err == 0
        tf = f.TimeStepByLSERKW2(tf, dt)
        to = o.timestep(to, dt)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert e <= 1e-10, e


def test_channel_body_force_with_cutoff():
    """The testcase source enters Ut before the filter (dg.f90:658-675)."""
    c = product_cfg(N=5, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1", OverintegrationType=1, NUnder=3,
                    kappa=1.4, R=1.0, Pr=0.72, mu0=1.0 / 2800.0, doTCSource=1, dpdx=-1.0)
    f, o, _ = channel_pair(c, nelems=(3, 4, 2))
    ut_f = f.DGTimeDerivative_weakForm(0.0)
    o.bulk_velocity()
    err = rel_err(ut_f, o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err
