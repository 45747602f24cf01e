"""Mortar interfaces on the GPU (k_mortar_pre, k_lift<MORTAR>, k_mortar_face; mortar.f90, fillmortar.t90)
against the oracle on the reference's own mortar meshes (tests/golden/hopr/).

- Ut parity at 1e-12 (as test_gpu_parity.py) on the periodic p_3D_mortar mesh (mortar types 1, 2, 3),
  the flipped h_3D_mortar meshes (type 3) and the run_basic/freestream_3D mortar box (types 1, 2, its
  Dirichlet sides replaced by adiabatic walls); Gauss and Gauss-Lobatto weak form, the Gauss-Lobatto and
  the Gauss split form, BR1 and BR2 lifting, lines of up to 11 nodes (the kernels whose arrays live in global scratch).
- the same on the library's synthetic mortar box (the mortar bench mesh) at 160 elements.
- a constant state is preserved on the periodic mortar meshes and a fluid at rest on the walled box.
- ten LSERK steps with the CFL time step agree with the oracle's (states at 1e-11), on the sine-wave
  convergence case of convtest/h_3D_mortar (no source term: the operator only).
- the adjoint (right-hand side and LSERK reverse sweep) against the oracle's exact JVP on mortar meshes.
"""
import os

import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, product_cfg, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
COMMON = dict(kappa=1.4, R=287.058, Pr=0.72, mu0=1e-3)
MESHES = ["CART_HEX_PERIODIC_MORTAR_002_mesh.h5", "CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5", "cartbox3D_mortar_mesh.h5"]


def _mesh(name):
    m0 = fmesh.read_hopr(os.path.join(HOPR, name))
    if name.startswith("cartbox"):
        return fmesh.read_hopr(os.path.join(HOPR, name), boundary={nm: (3, 0) for nm in m0.bc_names if nm != "inner"})
    return m0


def _state(x, seed, amp=0.1):
    return perturb_state(testcases.sine_wave_state(x, 0.0, (0.3, 0.3, 0.3)), seed=seed, amp=amp)


@pytest.mark.parametrize("name", MESHES)
@pytest.mark.parametrize("kw", [dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
                                dict(N=4, NodeType="gauss-lobatto", SplitDG="weak", Riemann="roe"),
                                dict(N=5, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix"),
                                dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2"),
                                dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc", Lifting="br2"),
                                dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix")])
def test_rhs_parity_mortar(name, kw):
    c = product_cfg(**kw, **COMMON)
    m = _mesh(name)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    # 5 % noise: with 10 % the Gauss split form's face entropy variable -rho/p, extrapolated from noisy nodes
    # at N=5, changes sign on FLIPPED_004 and EntropyToCons (a logarithm of it) is undefined, in both codes
    U0 = _state(f.elem_xgp(), seed=5, amp=0.05)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


@pytest.mark.parametrize("kw", [dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
                                dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix"),
                                dict(N=5, NodeType="gauss-lobatto", SplitDG="sd", Riemann="hllc")])
def test_rhs_parity_synthetic_mortar_box(kw):
    """The bench's mortar mesh (perturbed periodic mortar box, both big-side orientations) at a small size."""
    c = product_cfg(**kw, **COMMON)
    m = fmesh.mortar_box(4, perturb=0.05, seed=1)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.1, kappa=1.4, R=287.058), seed=7)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


@pytest.mark.parametrize("kw", [dict(N=8, NodeType="gauss", SplitDG="weak", Riemann="roe"),
                                dict(N=10, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
                                dict(N=9, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix")])
def test_rhs_parity_mortar_high_order(kw):
    c = product_cfg(**kw, **COMMON)
    m = _mesh("CART_HEX_PERIODIC_MORTAR_002_mesh.h5")
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = _state(f.elem_xgp(), seed=6)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


@pytest.mark.parametrize("name", MESHES)
def test_free_stream_mortar(name):
    c = product_cfg(N=4, NodeType="gauss", SplitDG="weak", Riemann="roe", **COMMON)
    f = Flexi(c, _mesh(name))
    x = f.elem_xgp()
    U = np.empty(x.shape[:-1] + (5,))
    if name.startswith("cartbox"):
        U[...] = [1.0, 0.0, 0.0, 0.0, 2.5]
    else:
        U[...] = [1.2, 0.3, -0.2, 0.5, 3.1]
    f.U = U
    Ut = f.DGTimeDerivative_weakForm(0.0)
    f.close()
    assert np.abs(Ut).max() <= 1e-12


def test_lserk_steps_mortar():
    c = product_cfg(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", CFLScale=0.9, DFLScale=0.9, **COMMON)
    m = _mesh("CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5")
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = testcases.sine_wave_state(f.elem_xgp(), 0.0, (0.3, 0.3, 0.3))
    f.U = U0
    o.set_state(U0)
    t_f = t_o = 0.0
    for _ in range(10):
        dt_f = f.CalcTimeStep()[0]
        dt_o = o.calc_timestep()[0]
        assert abs(dt_f / dt_o - 1.0) <= 1e-12
        t_f = f.TimeStepByLSERKW2(t_f, dt_f)
        t_o = o.timestep(t_o, dt_o)
    err = rel_err(f.U, o.get_state())
    f.close()
    assert err <= 1e-11, err


ADJ_MORTAR = {
    "p002_gauss3_weak_roe_br1": ("CART_HEX_PERIODIC_MORTAR_002_mesh.h5", dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe",
                                                                               Lifting="br1")),
    "flipped004_gl3_split_pi_roeef_br2": ("CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5",
                                          dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2")),
    "cartbox_gauss4_weak_hllc_br2": ("cartbox3D_mortar_mesh.h5", dict(N=4, NodeType="gauss", SplitDG="weak", Riemann="hllc", Lifting="br2")),
    "p002_gauss3_split_pi_roeef_br1": ("CART_HEX_PERIODIC_MORTAR_002_mesh.h5",
                                       dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1")),
}


@pytest.mark.parametrize("name", list(ADJ_MORTAR))
def test_adjoint_dot_product_mortar(name):
    """Adjoint on mortar meshes (transposed U_Mortar, Flux_Mortar of the numerical and the lifting fluxes, and
    the gradient interpolation): <J V, W> with J V the oracle's exact dual-number JVP against <V, J^T W> from
    the GPU adjoint, within 1e-11 of sum |JV_i W_i|; the viscosity-multiplier cotangent against a fourth-order
    Richardson quotient of <W, Ut> (1e-8)."""
    mesh_name, kw = ADJ_MORTAR[name]
    c = product_cfg(**kw, **COMMON)
    m = _mesh(mesh_name)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = _state(f.elem_xgp(), seed=11, amp=0.05)
    rng = np.random.default_rng(12)
    scale = rng.uniform(0.8, 1.2, f.n_elems)
    f.U = U0
    f.set_elem_mu_scale(scale)
    o.set_state(U0)
    o.set_mu_scale(scale)
    assert rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0)) <= 1e-12
    for _ in range(2):
        V = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
        W = rng.standard_normal(U0.shape)
        JV = o.jvp(V)
        JTW, mub = f.vjp_time_derivative(W)
        lhs, rhs = float((JV * W).sum()), float((V * JTW).sum())
        assert abs(lhs - rhs) <= 1e-11 * float(np.abs(JV * W).sum()), (lhs, rhs)
    ds = rng.standard_normal(f.n_elems)
    h = 1e-3

    def J(s):
        f.set_elem_mu_scale(s)
        return float((f.DGTimeDerivative_weakForm(0.0) * W).sum())

    d1 = (J(scale + h * ds) - J(scale - h * ds)) / (2 * h)
    d2 = (J(scale + 2 * h * ds) - J(scale - 2 * h * ds)) / (4 * h)
    rich = (4 * d1 - d2) / 3
    f.close()
    assert abs(float(mub @ ds) - rich) <= 1e-8 * abs(rich), (float(mub @ ds), rich)


def test_lserk_adjoint_mortar():
    """Seven LSERK steps reversed on a mortar mesh (fg_adjoint_forward / fg_adjoint_reverse) against the oracle's
    exact tangent of the same steps (dual numbers), 1e-10 of sum |JV_i w_i|."""
    c = product_cfg(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2", CFLScale=0.5, DFLScale=0.5, **COMMON)
    m = _mesh("CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5")
    f = Flexi(c, m)
    U0 = _state(f.elem_xgp(), seed=13, amp=0.05)
    f.U = U0
    dt = float(np.atleast_1d(f.CalcTimeStep()[0])[0])
    f.adjoint_forward(7, dt, 3)
    rng = np.random.default_rng(14)
    w = rng.standard_normal(U0.shape)
    Ub0, _ = f.adjoint_reverse(w)
    f.close()
    o = orc.Oracle(oracle_cfg(c), m)
    o.set_state(U0)
    V = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
    JV = o.jvp_solve(V, 7, dt)
    lhs, rhs = float((JV * w).sum()), float((Ub0 * V).sum())
    assert abs(lhs - rhs) <= 1e-10 * float(np.abs(JV * w).sum()), (lhs, rhs)


@pytest.mark.parametrize("name", ["CART_HEX_PERIODIC_MORTAR_002_mesh.h5", "cartbox3D_mortar_mesh.h5"])
def test_drop_in_mortar_mesh(name):
    """fg_set_mesh_mortar: FLEXI's own mesh arrays (SideToElem, ElemToSide, metrics, MortarType, MortarInfo,
    the small sides' metrics) as the oracle builds them; Ut at 1e-12 of the oracle."""
    c = product_cfg(N=4, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", **COMMON)
    m = _mesh(name)
    o = orc.Oracle(oracle_cfg(c), m)
    f = Flexi(c)
    f.set_mesh(o.mesh_iarray("SideToElem"), o.mesh_iarray("ElemToSide"), o.mesh_iarray("BC"), m.boundary_type, m.ref_state_prim,
               *(o.mesh_array(k) for k in ("Mf", "Mg", "Mh", "sJ", "NormVec", "TangVec1", "TangVec2", "SurfElem")),
               mortar_type=o.mesh_iarray("MortarType"), mortar_info=o.mesh_iarray("MortarInfo"))
    U0 = _state(o.mesh_array("Elem_xGP"), seed=8)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


@pytest.mark.parametrize("kw", [dict(N=5, NodeType="gauss", SplitDG="weak", OverintegrationType=1, NUnder=3),
                                dict(N=5, NodeType="gauss-lobatto", SplitDG="pi", OverintegrationType=2, NUnder=3)])
def test_overintegration_and_source_on_mortar_mesh(kw):
    """Overintegration (the filter of J u_t, overintegration.f90) and the exact-function source on a mortar
    mesh: Ut at t = 0.3 and five LSERK steps against the oracle."""
    c = product_cfg(Riemann="roeentropyfix", IniExactFunc=4, AdvVel=(0.3, 0.3, 0.3), **kw, **COMMON)
    m = _mesh("CART_HEX_PERIODIC_MORTAR_FLIPPED_004_mesh.h5")
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = _state(f.elem_xgp(), seed=9, amp=0.05)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.3), o.time_derivative(0.3))
    assert err <= 1e-12, err
    t_f = t_o = 0.3
    for _ in range(5):
        dt_f, dt_o = f.CalcTimeStep()[0], o.calc_timestep()[0]
        assert abs(dt_f / dt_o - 1.0) <= 1e-12
        t_f = f.TimeStepByLSERKW2(t_f, dt_f)
        t_o = o.timestep(t_o, dt_o)
    err = rel_err(f.U, o.get_state())
    f.close()
    assert err <= 1e-11, err


def test_ensemble_with_mortar_instance():
    """An ensemble of a mortar box and a conforming box (concatenate) gives each instance the time derivative
    of its own handle."""
    c = product_cfg(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", **COMMON)
    a, b = fmesh.mortar_box(2, perturb=0.05, seed=1), fmesh.tgv_box(2, ngeo=1, perturb=0.05, seed=2)
    fe = Flexi(c, fmesh.concatenate([a, b]))
    xe = fe.elem_xgp()
    Ue = perturb_state(testcases.tgv_state(xe, mach=0.1, kappa=1.4, R=287.058), seed=3)
    fe.U = Ue
    Ute = fe.DGTimeDerivative_weakForm(0.0)
    off = 0
    for m in (a, b):
        f = Flexi(c, m)
        f.U = Ue[off:off + m.n_elems]
        ut = f.DGTimeDerivative_weakForm(0.0)
        assert rel_err(Ute[off:off + m.n_elems], ut) <= 1e-14
        off += m.n_elems
        f.close()
    fe.close()
