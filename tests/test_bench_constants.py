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


@pytest.mark.parametrize("riemann", ["hllc", "roeentropyfix"])
def test_flops_per_dof_stage_match_oracle_count(riemann):
    bench = _bench()
    m = fmesh.tgv_box(4, ngeo=3, perturb=0.05)
    o = orc.Oracle(bench.oracle_config(riemann), m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    counted = o.flops_breakdown()
    for k, v in bench.flops_per_dof_stage(riemann).items():
        assert v == pytest.approx(counted[k], rel=2e-3), (k, v, counted[k])


def test_splitgauss_flops_per_dof_stage_match_oracle_count():
    bench = _bench()
    m = fmesh.tgv_box(4, ngeo=3, perturb=0.05)
    o = orc.Oracle(bench.oracle_config("roeentropyfix", "tgv-splitgauss"), m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    counted = o.flops_breakdown()
    for k, v in bench.flops_per_dof_stage("roeentropyfix", "tgv-splitgauss").items():
        assert v == pytest.approx(counted[k], rel=2e-3), (k, v, counted[k])


def test_oint_flops_per_dof_stage_match_oracle_count():
    bench = _bench()
    m = fmesh.tgv_box(2, ngeo=3, perturb=0.05)
    o = orc.Oracle(bench.oracle_config("roeentropyfix", "tgv-oint"), m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    counted = o.flops_breakdown()
    for k, v in bench.flops_per_dof_stage("roeentropyfix", "tgv-oint").items():
        assert v == pytest.approx(counted[k], rel=2e-3), (k, v, counted[k])


def test_mortar_flops_per_dof_stage_match_oracle_count():
    bench = _bench()
    m = fmesh.mortar_box(2, perturb=0.05)
    o = orc.Oracle(bench.oracle_config("roeentropyfix", "tgv-mortar"), m)
    o.set_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.1, kappa=1.4, R=71.42857))
    counted = o.flops_breakdown()
    for k, v in bench.flops_per_dof_stage("roeentropyfix", "tgv-mortar").items():
        assert v == pytest.approx(counted[k], rel=2e-3), (k, v, counted[k])
