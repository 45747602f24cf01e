"""Adjoint of the right-hand side (fg_vjp_time_derivative) against the oracle's Jacobian-vector products.

Cases: the weak form and every split form (SD, PI, MO, DU, KG, CH, IR) on Gauss-Lobatto nodes (the shuffle-pair kernel
for PI on lines of 2, 4 or 8 nodes, the per-node kernel otherwise) and on Gauss nodes (entropy-variable prolongation and split-Gauss
surface term transposed), every Riemann solver of riemann.f90, BR1/BR2, both overintegration types, walls.

Dot-product test <J V, W> = <V, J^T W>: J V comes from the oracle, exactly by its dual-number
instantiation of the restated algorithm and approximately by the matrix-free finite difference of the
reference's implicit solver (src/implicit/implicit.f90:MatrixVector, FD_Order 2); J^T W comes from the
GPU adjoint kernels. Bars: exact JVP within 1e-11 of the sum of |JV_i W_i| (round-off only), FD JVP
within 1e-8 relative. The viscosity-multiplier cotangent is checked against a central difference of
<W, Ut> in a random direction of the multipliers (1e-8 relative), and the forward with random
multipliers against the oracle (1e-12, as all forward parity tests)."""
import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

CASES = {
    "gauss3_weak_roeef_br1": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1"), "tgv"),
    "gauss5_weak_roe_br2": (dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2", etaBR2=2.5), "tgv"),
    "gl3_weak_lf_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="weak", Riemann="lf", Lifting="br1"), "tgv"),
    "gl7_split_pi_roe_br1": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1"), "tgv"),
    "gl7_split_pi_roeef_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"), "tgv"),
    "gl3_split_pi_lf_br2": (dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="lf", Lifting="br2"), "tgv"),
    # HLLC: the surface flux of the N=7 TGV benchmark
    "gl7_split_pi_hllc_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc", Lifting="br2"), "tgv"),
    "gauss3_weak_hllc_br1": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hllc", Lifting="br1"), "tgv"),
    # overintegration (the transposed filter): modal cut-off and conservative cut-off
    "gauss5_weak_roeef_br1_cutoff": (dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1",
                                          OverintegrationType=1, NUnder=3), "tgv"),
    "gl7_split_pi_roeef_br2_conscutoff": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2",
                                               OverintegrationType=2, NUnder=4), "tgv"),
    "gauss3_split_pi_roeef_br1_conscutoff": (dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1",
                                                  OverintegrationType=2, NUnder=2), "tgv"),
    # split form on Gauss nodes (entropy-variable prolongation, split-Gauss surface term): the discretisation of the
    # reference's tgv/splitGauss regression at N=5, and SD at N=3 with BR2
    "gauss5_split_pi_roeef_br1": (dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1"), "tgv"),
    "gauss3_split_sd_hllc_br2": (dict(N=3, NodeType="gauss", SplitDG="sd", Riemann="hllc", Lifting="br2"), "tgv"),
    "gauss4_split_pi_lf_br2": (dict(N=4, NodeType="gauss", SplitDG="pi", Riemann="lf", Lifting="br2"), "tgv"),
    # split form on Gauss-Lobatto lines the shuffle-pair kernel does not take: SD, and PI with odd node counts
    "gl3_split_sd_roe_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="sd", Riemann="roe", Lifting="br1"), "tgv"),
    "gl4_split_pi_roeef_br2": (dict(N=4, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"), "tgv"),
    # the other Riemann solvers: HLL, HLLE, HLLEM (physical fluxes, Roe or Einfeldt signal speeds), RoeL2 (Mach-scaled jumps),
    # RoeEntropyGShockFix (wave speeds limited by c / RiemannPhiFactor), and the split form's flux average
    "gauss3_weak_hll_br1": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hll", Lifting="br1"), "tgv"),
    "gl3_weak_hlle_br2": (dict(N=3, NodeType="gauss-lobatto", SplitDG="weak", Riemann="hlle", Lifting="br2"), "tgv"),
    "gauss4_weak_hllem_br1": (dict(N=4, NodeType="gauss", SplitDG="weak", Riemann="hllem", Lifting="br1"), "tgv"),
    "gl3_split_pi_hllem_br2": (dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllem", Lifting="br2"), "tgv"),
    "gauss3_weak_roel2_br1": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roel2", Lifting="br1"), "tgv"),
    "gl7_split_pi_roel2_br1": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roel2", Lifting="br1"), "tgv"),
    "gauss3_weak_gshock_br2": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropygshockfix", Lifting="br2"), "tgv"),
    "gl3_split_sd_gshock_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="sd", Riemann="roeentropygshockfix", Lifting="br1"), "tgv"),
    "gl7_split_pi_avg_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="avg", Lifting="br2"), "tgv"),
    "gauss3_split_sd_avg_br1": (dict(N=3, NodeType="gauss", SplitDG="sd", Riemann="avg", Lifting="br1"), "tgv"),
    "channel_gauss3_weak_hlle_br2": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hlle", Lifting="br2"), "channel"),
    # the split fluxes MO, DU, KG (per-node kernel; on Gauss nodes with the entropy-variable prolongation) with the surface
    # fluxes of both kernel variants
    "gl3_split_mo_roe_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="mo", Riemann="roe", Lifting="br1"), "tgv"),
    "gl4_split_du_lf_br2": (dict(N=4, NodeType="gauss-lobatto", SplitDG="du", Riemann="lf", Lifting="br2"), "tgv"),
    "gl7_split_kg_hllc_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="kg", Riemann="hllc", Lifting="br2"), "tgv"),
    "gauss3_split_kg_roeef_br1": (dict(N=3, NodeType="gauss", SplitDG="kg", Riemann="roeentropyfix", Lifting="br1"), "tgv"),
    "gauss4_split_du_avg_br1": (dict(N=4, NodeType="gauss", SplitDG="du", Riemann="avg", Lifting="br1"), "tgv"),
    "gl3_split_mo_roel2_br2": (dict(N=3, NodeType="gauss-lobatto", SplitDG="mo", Riemann="roel2", Lifting="br2"), "tgv"),
    "channel_gauss3_split_mo_hll_br1": (dict(N=3, NodeType="gauss", SplitDG="mo", Riemann="hll", Lifting="br1"), "channel"),
    # the entropy-conserving split fluxes CH and IR (logarithmic means) and the CH and IR surface fluxes
    "gl3_split_ch_ch_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="ch", Riemann="ch", Lifting="br1"), "tgv"),
    "gl4_split_ir_roeef_br2": (dict(N=4, NodeType="gauss-lobatto", SplitDG="ir", Riemann="roeentropyfix", Lifting="br2"), "tgv"),
    "gl7_split_ch_lf_br2": (dict(N=7, NodeType="gauss-lobatto", SplitDG="ch", Riemann="lf", Lifting="br2"), "tgv"),
    "gauss3_split_ir_ir_br1": (dict(N=3, NodeType="gauss", SplitDG="ir", Riemann="ir", Lifting="br1"), "tgv"),
    "gauss4_split_pi_ir_br2": (dict(N=4, NodeType="gauss", SplitDG="pi", Riemann="ir", Lifting="br2"), "tgv"),
    "gl3_split_mo_ch_br1": (dict(N=3, NodeType="gauss-lobatto", SplitDG="mo", Riemann="ch", Lifting="br1"), "tgv"),
    "channel_gauss3_weak_roe_br1": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1"), "channel"),
    "channel_gauss3_split_pi_roe_br2": (dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roe", Lifting="br2"), "channel"),
    "channel_gl7_split_pi_roe_br1": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1"), "channel"),
    "channel_gl3_split_pi_roeef_br2_adiabatic": (dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"),
                                                 "adiabatic"),
}


def _setup(name, seed=0):
    kw, kind = CASES[name]
    c = make_config(mu0=5e-3, R=1.0 if kind != "tgv" else 71.42857, **kw)
    if kind == "tgv":
        m = fmesh.tgv_box(3, ngeo=2, perturb=0.05, seed=seed)
    elif kind == "channel":
        m = fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2, t_wall=1.0)
    else:
        m = fmesh.cartesian_box((3, 3, 2), (0.0, -1.0, 0.0), (2.0, 1.0, 1.0), ngeo=1, periodic=(True, False, True), wall_bc=(3, 1),
                                ref_state_prim=np.array([[1.0, 0.0, 0.0, 0.0, 1.0, 1.0]]))
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    x = f.elem_xgp()
    if kind == "tgv":
        U = testcases.tgv_state(x, mach=0.3, kappa=c.kappa, R=c.R)
    else:
        U = testcases.channel_state(x, mach=0.3, kappa=c.kappa, R=c.R, t_wall=1.0, noise=0.0, seed=seed)
    U = perturb_state(U, seed=seed + 7, amp=0.05)
    rng = np.random.default_rng(seed + 100)
    scale = rng.uniform(0.8, 1.2, f.n_elems)
    f.U = U
    f.set_elem_mu_scale(scale)
    o.set_state(U)
    o.set_mu_scale(scale)
    return f, o, U, scale, rng


@pytest.mark.parametrize("name", list(CASES))
def test_forward_with_viscosity_multipliers(name):
    f, o, U, scale, rng = _setup(name)
    assert rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative()) <= 1e-12


@pytest.mark.parametrize("name", list(CASES))
def test_dot_product_against_exact_jvp(name):
    f, o, U, scale, rng = _setup(name)
    for k in range(2):
        V = rng.standard_normal(U.shape) * np.abs(U).max(axis=(0, 1, 2, 3))
        W = rng.standard_normal(U.shape)
        JV = o.jvp(V)
        JTW, _ = f.vjp_time_derivative(W)
        lhs = float((JV * W).sum())
        rhs = float((V * JTW).sum())
        scale_ = float(np.abs(JV * W).sum())
        assert abs(lhs - rhs) <= 1e-11 * scale_, (k, lhs, rhs, abs(lhs - rhs) / scale_)


@pytest.mark.parametrize("name", ["gauss3_weak_roeef_br1", "gl7_split_pi_roe_br1", "channel_gl7_split_pi_roe_br1",
                                  "gauss5_split_pi_roeef_br1"])
def test_dot_product_against_reference_fd_jvp(name):
    f, o, U, scale, rng = _setup(name, seed=1)
    V = rng.standard_normal(U.shape) * np.abs(U).max(axis=(0, 1, 2, 3))
    W = rng.standard_normal(U.shape)
    JV = o.fd_jvp(V, fd_order=2, eps_method=1)
    JTW, _ = f.vjp_time_derivative(W)
    lhs, rhs = float((JV * W).sum()), float((V * JTW).sum())
    assert abs(lhs - rhs) <= 1e-8 * float(np.abs(JV * W).sum()), (lhs, rhs)


@pytest.mark.parametrize("name", ["gauss3_weak_roeef_br1", "gl7_split_pi_roeef_br2", "channel_gauss3_weak_roe_br1",
                                  "gauss3_split_sd_hllc_br2"])
def test_viscosity_multiplier_cotangent(name):
    f, o, U, scale, rng = _setup(name, seed=2)
    W = rng.standard_normal(U.shape)
    _, mub = f.vjp_time_derivative(W)
    ds = rng.standard_normal(f.n_elems)
    h = 1e-3  # fourth-order Richardson quotient: truncation ~h^4, round-off / h ~1e-13

    def J(s):
        f.set_elem_mu_scale(s)
        return float((f.DGTimeDerivative_weakForm(0.0) * W).sum())

    fd = (J(scale + h * ds) - J(scale - h * ds)) / (2 * h)
    fd2 = (J(scale + 2 * h * ds) - J(scale - 2 * h * ds)) / (4 * h)
    rich = (4 * fd - fd2) / 3
    assert abs(float(mub @ ds) - rich) <= 1e-8 * abs(rich), (float(mub @ ds), rich)


def test_vjp_rejects_unsupported():
    c = make_config(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", doWeakLifting=1)
    f = Flexi(c, fmesh.tgv_box(2))
    f.U = testcases.tgv_state(f.elem_xgp(), mach=0.1)
    with pytest.raises(Exception, match="strong, non-conservative lifting"):
        f.vjp_time_derivative(np.zeros(f.ushape))


@pytest.mark.parametrize("name", ["gauss3_weak_roeef_br1", "gl7_split_pi_roe_br1", "channel_gl7_split_pi_roe_br1"])
@pytest.mark.parametrize("fd_order,eps_method,tol_exact", [(2, 1, 1e-5), (1, 2, 1e-3)])
def test_fd_jvp_on_gpu(name, fd_order, eps_method, tol_exact):
    """fg_jvp_time_derivative (the reference's MatrixVector finite difference, on the GPU) against the exact
    JVP in the 2-norm, within the recipe's own accuracy (1e-5 central, 1e-3 one-sided: the reference scales
    the step by the global norm of V, so each entry moves by ~1e-10 and round-off over the step dominates
    single entries), and at most 10x the error of the same recipe on the oracle; the state is unchanged."""
    f, o, U, scale, rng = _setup(name, seed=3)
    V = rng.standard_normal(U.shape) * np.abs(U).max(axis=(0, 1, 2, 3))
    JVg = f.jvp_time_derivative(V, fd_order=fd_order, eps_method=eps_method)
    assert np.array_equal(f.U, U)
    JVx = o.jvp(V)
    JVo = o.fd_jvp(V, fd_order=fd_order, eps_method=eps_method)
    nrm = np.linalg.norm(JVx)
    err_g, err_o = np.linalg.norm(JVg - JVx) / nrm, np.linalg.norm(JVo - JVx) / nrm
    assert err_g <= tol_exact, err_g
    assert err_g <= 10 * err_o + 1e-12, (err_g, err_o)
