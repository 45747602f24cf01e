"""The lifting options of the oracle (lifting.f90: doWeakLifting, doConservativeLifting; lifting_volint.t90,
lifting_br1.t90) pinned by the identities the scheme satisfies. On affine elements the conservative volume
part equals the non-conservative one (constant metrics), and the weak form equals the strong form by
summation by parts, provided the face values the strong form subtracts are the interpolated volume values:
always on Gauss-Lobatto nodes (face nodes are volume nodes), on Gauss nodes when the conservative state is
a polynomial of degree <= N (the lifting variables at the faces come from the prolonged conservative
state). So the time derivative of all forms agrees to round-off there; on curved elements the conservative
and weak forms differ from the strong form by aliasing only (small, not round-off).
"""
import numpy as np
import pytest

from _cases import perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from oracle import oracle as orc

BASE = dict(riemann=33, riemannBC=-1, splitDG=-1, etaBR2=2.0, etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=5e-3,
            CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0)


def _ut(mesh, node_type, lifting, weak, cons, seed=3):
    o = orc.Oracle(dict(BASE, N=4, nodeType=node_type, lifting=lifting, weakLifting=weak, consLifting=cons), mesh)
    x = o.mesh_array("Elem_xGP")
    o.set_state(perturb_state(testcases.tgv_state(x, mach=0.3, kappa=1.4, R=71.42857), seed=seed, amp=0.05))
    return o.time_derivative(0.0)


@pytest.mark.parametrize("node_type", [orc.NT_GAUSS, orc.NT_GL])
def test_lifting_forms_agree_on_affine_elements(node_type):
    m = fmesh.tgv_box(3, ngeo=1)
    ref = _ut(m, node_type, 1, 0, 0)
    scale = np.abs(ref).max()
    forms = ((0, 1), (1, 0)) if node_type == orc.NT_GL else ((0, 1),)
    for weak, cons in forms:
        assert np.abs(_ut(m, node_type, 1, weak, cons) - ref).max() <= 1e-12 * scale, (weak, cons)
    assert np.abs(_ut(m, node_type, 2, 0, 1) - _ut(m, node_type, 2, 0, 0)).max() <= 1e-12 * scale
    if node_type == orc.NT_GAUSS:  # noisy state: the face primitives are not the interpolated ones
        assert np.abs(_ut(m, node_type, 1, 1, 0) - ref).max() > 1e-6 * scale


def test_weak_equals_strong_lifting_on_gauss_nodes_for_polynomial_states():
    """Walls at y = +-1 (isothermal), state linear in y (rho = 1): E is quadratic, so at N = 4 the prolonged
    conservative state and the face primitives are exact and weak = strong lifting to round-off."""
    m = fmesh.cartesian_box((3, 3, 3), (-1.0,) * 3, (1.0,) * 3, periodic=(True, False, True), wall_bc=(4, 1),
                            ref_state_prim=[[1.0, 0.0, 0.0, 0.0, 1.0, 1.0 / 71.42857]])
    uts = []
    for weak, cons in ((0, 0), (1, 0), (0, 1)):
        o = orc.Oracle(dict(BASE, N=4, nodeType=orc.NT_GAUSS, lifting=1, weakLifting=weak, consLifting=cons), m)
        x = o.mesh_array("Elem_xGP")
        y = x[..., 1]
        U = np.zeros(x.shape[:-1] + (5,))
        vel = np.stack([0.1 + 0.2 * y, 0.05 * y, -0.1 * y], axis=-1)
        p = 1.0 + 0.3 * y
        U[..., 0] = 1.0
        U[..., 1:4] = vel
        U[..., 4] = p / 0.4 + 0.5 * (vel ** 2).sum(-1)
        o.set_state(U)
        uts.append(o.time_derivative(0.0))
    scale = np.abs(uts[0]).max()
    assert np.abs(uts[1] - uts[0]).max() <= 1e-12 * scale
    assert np.abs(uts[2] - uts[0]).max() <= 1e-12 * scale


@pytest.mark.parametrize("node_type", [orc.NT_GAUSS, orc.NT_GL])
def test_lifting_forms_differ_by_aliasing_on_curved_elements(node_type):
    m = fmesh.tgv_box(3, ngeo=3, perturb=0.1, seed=2)
    ref = _ut(m, node_type, 1, 0, 0)
    scale = np.abs(ref).max()
    for weak, cons in ((0, 1), (1, 0)):
        d = np.abs(_ut(m, node_type, 1, weak, cons) - ref).max() / scale
        assert 1e-12 < d < 1e-2, (weak, cons, d)
