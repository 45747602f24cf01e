"""Pins the algorithmic flop counts bench.py uses for the roofline to the oracle's flop-counting scalar
(every +,-,*,/,sqrt = 1 flop) on the benchmark discretisation."""
import importlib.util
import os

import pytest

from flexi_gb300 import mesh as fmesh, testcases
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_flops_per_dof_stage_match_oracle_count():
    bench = _bench()
    cfg = dict(N=7, nodeType=2, riemann=33, riemannBC=-1, lifting=2, weakLifting=0, consLifting=0, splitDG=4, etaBR2=2.0, etaBR2_wall=-1.0,
               kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.8, DFLScale=0.8, doTCSource=0, dpdx=-1.0)
    m = fmesh.tgv_box(4, ngeo=3, perturb=0.05)
    o = orc.Oracle(cfg, m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    counted = o.flops_breakdown()
    for k, v in bench.FLOPS_PER_DOF_STAGE.items():
        assert v == pytest.approx(counted[k], rel=2e-3), (k, v, counted[k])
