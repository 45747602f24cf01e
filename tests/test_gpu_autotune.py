"""Launch-shape autotuner (fg_autotune / fg_set_launch_shapes): every shape gives the same result.

The shapes only regroup elements into CTAs (and side points into blocks), so the time derivative and a
few time steps are bitwise identical for every combination; the tuner reports a time for every
candidate of the order (NaN where none exists) and leaves the state unchanged."""
import itertools

import numpy as np
import pytest

from _cases import perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config

pytestmark = pytest.mark.gpu

CASES = {"gauss5": (dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1"), (1, 2)),
         "gauss3": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2"), (2, 4)),
         "gl7_split": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"), (1,))}


@pytest.mark.parametrize("name", list(CASES))
def test_launch_shapes_do_not_change_results(name):
    kw, epbs = CASES[name]
    c = make_config(mu0=2e-3, R=71.42857, **kw)
    f = Flexi(c, fmesh.tgv_box(3, ngeo=2, perturb=0.05, seed=1))
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.2, kappa=c.kappa, R=c.R), seed=2)
    f.U = U0
    ref = f.DGTimeDerivative_weakForm(0.0)
    f.TimeDisc(3)
    ref_steps = f.U
    for ep, el, ev in itertools.product(epbs, epbs, epbs):
        for blk in (64, 128, 256):
            f.set_launch_shapes(ep, el, ev, blk)
            f.U = U0
            assert np.array_equal(f.DGTimeDerivative_weakForm(0.0), ref), (ep, el, ev, blk)
    f.U = U0
    rep = f.autotune(reps=3)
    assert np.array_equal(f.U, U0)
    t = rep["ms_per_launch"]
    assert all(t[k] is not None and t[k] > 0 for k in ("flux_64", "flux_128", "flux_256"))
    if len(epbs) > 1:
        assert all(t[k] is not None and t[k] > 0 for k in ("prep_default", "prep_alt", "lift_default", "lift_alt", "vol_default", "vol_alt"))
    else:
        assert t["prep_alt"] is None
    f.TimeDisc(3)
    assert np.array_equal(f.U, ref_steps)
