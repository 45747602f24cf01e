"""Overintegration in the CPU oracle (src/dg/overintegration.f90): properties that hold independently of
the regression data (tests/test_oracle_tgv.py pins the modal cut-off against tgv/oInt).

- The cut-off filter is a projection: filtering the state twice equals filtering it once (1e-13).
- On an affine mesh the Jacobian is constant, so the conservative cut-off (project J u_t to NUnder, multiply
  by 1/J there, interpolate back) equals the plain cut-off followed by ApplyJacobian (1e-12).
- NUnder >= N switches the conservative cut-off off (overintegration.f90:139-141): the time derivative is
  the one without overintegration, bit for bit.
"""
import numpy as np
import pytest

from _cases import perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from oracle import oracle as orc

BASE = dict(N=5, nodeType=orc.NT_GAUSS, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=-1,
            etaBR2=2.0, etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=5e-3, CFLScale=0.9, DFLScale=0.9,
            doTCSource=0, dpdx=-1.0)


def _oracle(mesh, **kw):
    o = orc.Oracle(dict(BASE, **kw), mesh)
    U = perturb_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), mach=0.2, kappa=1.4, R=71.42857), seed=3, amp=0.05)
    o.set_state(U)
    return o, U


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_cutoff_filter_is_a_projection():
    m = fmesh.tgv_box(2, ngeo=2, perturb=0.1, seed=1)
    o, U = _oracle(m, overintType=1, NUnder=3)
    o.overintegrate_state()
    once = o.get_state()
    o.overintegrate_state()
    assert _rel(o.get_state(), once) <= 1e-13
    assert _rel(once, U) > 1e-4  # the filter removed modes 4 and 5


@pytest.mark.parametrize("node_type", [orc.NT_GAUSS, orc.NT_GL])
def test_conservative_cutoff_equals_cutoff_on_affine_mesh(node_type):
    m = fmesh.tgv_box(2, ngeo=1)
    o1, _ = _oracle(m, nodeType=node_type, overintType=1, NUnder=3)
    o2, _ = _oracle(m, nodeType=node_type, overintType=2, NUnder=3)
    assert _rel(o2.time_derivative(0.0), o1.time_derivative(0.0)) <= 1e-12
    o1.overintegrate_state()
    o2.overintegrate_state()
    assert _rel(o2.get_state(), o1.get_state()) <= 1e-12


def test_conservative_cutoff_off_for_nunder_not_below_n():
    m = fmesh.tgv_box(2, ngeo=2, perturb=0.1, seed=2)
    o0, _ = _oracle(m)
    o2, _ = _oracle(m, overintType=2, NUnder=5)
    assert np.array_equal(o2.time_derivative(0.0), o0.time_derivative(0.0))
