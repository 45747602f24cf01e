"""All six low-storage schemes of TimeStepByLSERKW2 on the GPU against the oracle (timestep.f90:82-152).

For every TimeDiscMethod: the CALCTIMESTEP step (CFLScaleAlpha / RelativeDFL of the scheme) equals the
oracle's, and five steps of the scheme with the time-dependent source of exact function 4 (stage times
t + RKc dt) agree with the oracle's at 1e-11, on Gauss and Gauss-Lobatto nodes; the captured step graph
(fg_run) of the 14-stage scheme equals single steps.
"""
import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, product_cfg, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

ADV = (0.3, 0.2, 0.1)


def _cfg(code, node_type):
    return product_cfg(N=4, NodeType=node_type, SplitDG="weak" if node_type == "gauss" else "pi", Riemann="roeentropyfix",
                       Lifting="br1", kappa=1.4, R=287.058, Pr=0.72, mu0=1e-3, CFLScale=0.9, DFLScale=0.9, IniExactFunc=4, AdvVel=ADV,
                       TimeDiscMethod=code)


@pytest.mark.parametrize("node_type", ["gauss", "gauss-lobatto"])
@pytest.mark.parametrize("code", range(6))
def test_scheme_parity(code, node_type):
    c = _cfg(code, node_type)
    m = fmesh.cartesian_box((3, 3, 3), (-1,) * 3, (1,) * 3, ngeo=2, mapping=lambda x, y, z: (x + 0.05 * np.sin(np.pi * y), y, z))
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = perturb_state(testcases.sine_wave_state(f.elem_xgp(), 0.0, ADV), seed=4, amp=0.05)
    f.U = U0
    o.set_state(U0)
    t_f = t_o = 0.1
    for _ in range(5):
        dt_f, dt_o = f.CalcTimeStep()[0], o.calc_timestep()[0]
        assert abs(dt_f / dt_o - 1.0) <= 1e-12
        t_f = f.TimeStepByLSERKW2(t_f, dt_f)
        t_o = o.timestep(t_o, dt_o)
    err = rel_err(f.U, o.get_state())
    f.close()
    assert err <= 1e-11, err


def test_captured_graph_fourteen_stages():
    c = _cfg(2, "gauss")
    m = fmesh.cartesian_box((3, 3, 3), (-1,) * 3, (1,) * 3)
    f, g = Flexi(c, m), Flexi(c, m)
    U0 = testcases.sine_wave_state(f.elem_xgp(), 0.0, ADV)
    f.U = U0
    g.U = U0
    t_f = f.TimeDisc(4)[0]
    t_g = 0.0
    for _ in range(4):
        t_g = g.TimeStepByLSERKW2(t_g, g.CalcTimeStep()[0])
    assert abs(t_f - t_g) <= 1e-15 * t_g
    err = rel_err(f.U, g.U)
    f.close()
    g.close()
    assert err <= 1e-13, err
