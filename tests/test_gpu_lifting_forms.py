"""The lifting options doWeakLifting (BR1) and doConservativeLifting (BR1, BR2) on the GPU (k_lift's
conservative volume part, lifting_volint.t90:Lifting_VolInt_Conservative with D_T or D_Hat_T; the weak
surface signs of lifting_fillflux.t90 / lifting_br1.t90) against the oracle: Ut at 1e-12 and five LSERK
steps at 1e-11 on curved periodic boxes, the isothermal-wall channel, a mortar mesh and lines of 11 nodes
(the global-scratch variant)."""
import os

import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, product_cfg, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
COMMON = dict(kappa=1.4, R=71.42857, Pr=0.72, mu0=5e-3, Riemann="roeentropyfix")
CASES = {
    "gauss3_weak_br1_weaklift": (dict(N=3, NodeType="gauss", SplitDG="weak", Lifting="br1", doWeakLifting=1), "tgv"),
    "gauss5_weak_br1_conslift": (dict(N=5, NodeType="gauss", SplitDG="weak", Lifting="br1", doConservativeLifting=1), "tgv"),
    "gl4_split_pi_br1_weaklift": (dict(N=4, NodeType="gauss-lobatto", SplitDG="pi", Lifting="br1", doWeakLifting=1), "tgv"),
    "gl7_split_pi_br2_conslift": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Lifting="br2", doConservativeLifting=1), "tgv"),
    "gauss4_weak_br1_weaklift_channel": (dict(N=4, NodeType="gauss", SplitDG="weak", Lifting="br1", doWeakLifting=1), "channel"),
    "gl4_weak_br1_weaklift_mortar": (dict(N=4, NodeType="gauss-lobatto", SplitDG="weak", Lifting="br1", doWeakLifting=1), "mortar"),
    "gauss10_weak_br1_conslift": (dict(N=10, NodeType="gauss", SplitDG="weak", Lifting="br1", doConservativeLifting=1), "tgv2"),
}


def _pair(name):
    kw, kind = CASES[name]
    c = product_cfg(**kw, **COMMON)
    if kind == "channel":
        m = fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2, t_wall=1.0, rho_wall=1.0, p_wall=71.42857)
    elif kind == "mortar":
        m = fmesh.read_hopr(os.path.join(HOPR, "CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5"))
    else:
        m = fmesh.tgv_box(2 if kind == "tgv2" else 3, ngeo=3, perturb=0.1, seed=4)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    x = f.elem_xgp()
    if kind == "channel":
        U0 = testcases.channel_state(x, mach=0.1, kappa=1.4, R=71.42857, t_wall=1.0, noise=0.05, seed=2)
    else:
        U0 = perturb_state(testcases.tgv_state(x, mach=0.3, kappa=1.4, R=71.42857), seed=6, amp=0.05)
    f.U = U0
    o.set_state(U0)
    return f, o


@pytest.mark.parametrize("name", list(CASES))
def test_rhs_and_steps(name):
    f, o = _pair(name)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    assert err <= 1e-12, err
    t_f = t_o = 0.0
    for _ in range(5):
        dt_f, dt_o = f.CalcTimeStep()[0], o.calc_timestep()[0]
        assert abs(dt_f / dt_o - 1.0) <= 1e-12
        t_f = f.TimeStepByLSERKW2(t_f, dt_f)
        t_o = o.timestep(t_o, dt_o)
    err = rel_err(f.U, o.get_state())
    f.close()
    assert err <= 1e-11, err
