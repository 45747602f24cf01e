"""GPU parity of libflexigpu.so against the CPU oracle (restatement of FLEXI's operator).

Bars (FP64 throughout): time derivative Ut after one DGTimeDerivative_weakForm within 1e-12 (max abs
error per conservative variable, normalised by that variable's max |Ut|); state after RK steps within
1e-10 (same norm). Results differ from the oracle only by floating-point summation order."""
import numpy as np
import pytest

from _cases import channel_pair, product_cfg, rel_err, tgv_pair
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

UT_TOL = 1e-12
STATE_TOL = 1e-10

RHS_CASES = {
    # plain method, small: TGV, N=3 Gauss, weak form, Roe, BR1
    "c1_gauss3_weak_roe_br1": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1"),
    "gauss3_weak_lf": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="lf"),
    "gauss3_weak_hllc": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hllc"),
    "gauss3_weak_roeef": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
    "gauss3_weak_br2": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2", etaBR2=2.5),
    "gauss5_weak_roeef": dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
    "gauss1_weak": dict(N=1, NodeType="gauss", SplitDG="weak", Riemann="roe"),
    "gauss2_weak": dict(N=2, NodeType="gauss", SplitDG="weak", Riemann="roe"),
    "gauss4_weak": dict(N=4, NodeType="gauss", SplitDG="weak", Riemann="roe"),
    "gauss6_weak": dict(N=6, NodeType="gauss", SplitDG="weak", Riemann="roe"),
    "gauss7_weak": dict(N=7, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
    "gl3_weak_roe": dict(N=3, NodeType="gauss-lobatto", SplitDG="weak", Riemann="roe"),
    "gl5_weak_lf": dict(N=5, NodeType="gauss-lobatto", SplitDG="weak", Riemann="lf"),
    # split forms (Gauss-Lobatto)
    "gl7_split_pi_roeef_br1": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1"),
    "gl7_split_pi_roeef_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"),
    "gl7_split_pi_hllc_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc", Lifting="br2"),
    "gl7_split_sd_roe": dict(N=7, NodeType="gauss-lobatto", SplitDG="sd", Riemann="roe"),
    "gl3_split_pi_lf": dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="lf"),
    "gl1_split_pi": dict(N=1, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe"),
    # split forms on Gauss-Lobatto lines of 3, 5, 6, 7 nodes (k_vol_split_gen)
    "gl2_split_pi_roe": dict(N=2, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe"),
    "gl4_split_sd_lf": dict(N=4, NodeType="gauss-lobatto", SplitDG="sd", Riemann="lf"),
    "gl5_split_pi_roeef_br2": dict(N=5, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"),
    "gl6_split_pi_hllc": dict(N=6, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc"),
    # split forms on Gauss nodes: entropy-variable prolongation and the split-Gauss surface integral
    "gauss5_split_pi_roeef_br1": dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1"),
    "gauss5_split_pi_hllc_br2": dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="hllc", Lifting="br2"),
    "gauss3_split_pi_roe_br2": dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roe", Lifting="br2", etaBR2=2.5),
    "gauss3_split_sd_lf": dict(N=3, NodeType="gauss", SplitDG="sd", Riemann="lf"),
    "gauss1_split_pi": dict(N=1, NodeType="gauss", SplitDG="pi", Riemann="roe"),
    "gauss2_split_pi_roeef": dict(N=2, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix"),
    "gauss4_split_sd_roe": dict(N=4, NodeType="gauss", SplitDG="sd", Riemann="roe"),
    "gauss6_split_pi_lf": dict(N=6, NodeType="gauss", SplitDG="pi", Riemann="lf"),
    "gauss7_split_pi_roeef": dict(N=7, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix"),
    # lines of 9..12 nodes: several nodes per thread; per-element arrays in the global scratch where they
    # exceed shared memory
    "gauss8_weak_roe_br2": dict(N=8, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br2"),
    "gl9_weak_lf": dict(N=9, NodeType="gauss-lobatto", SplitDG="weak", Riemann="lf"),
    "gauss11_weak_roeef_br1": dict(N=11, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1"),
    "gl11_split_pi_roeef_br2": dict(N=11, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"),
    "gauss8_split_pi_hllc": dict(N=8, NodeType="gauss", SplitDG="pi", Riemann="hllc"),
    "gauss10_split_sd_roe_br2": dict(N=10, NodeType="gauss", SplitDG="sd", Riemann="roe", Lifting="br2"),
    # the other SplitDG fluxes (MO, DU, KG, CH, IR) and Riemann solvers (RoeL2, RoeEntropyGShockFix, HLL, HLLE, HLLEM, and the
    # split-only CH, IR, avg) of splitflux.f90 / riemann.f90
    "gl7_split_mo_roe": dict(N=7, NodeType="gauss-lobatto", SplitDG="mo", Riemann="roe"),
    "gl7_split_du_roel2_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="du", Riemann="roel2", Lifting="br2"),
    "gl7_split_kg_gshock": dict(N=7, NodeType="gauss-lobatto", SplitDG="kg", Riemann="roeentropygshockfix", RiemannPhiFactor=3.0),
    "gl7_split_ch_ch_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="ch", Riemann="ch", Lifting="br2"),
    "gl7_split_ir_ir": dict(N=7, NodeType="gauss-lobatto", SplitDG="ir", Riemann="ir"),
    "gl7_split_pi_avg": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="avg"),
    "gl7_split_pi_hllem": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllem"),
    "gl5_split_kg_avg": dict(N=5, NodeType="gauss-lobatto", SplitDG="kg", Riemann="avg"),
    "gl4_split_ch_roeef": dict(N=4, NodeType="gauss-lobatto", SplitDG="ch", Riemann="roeentropyfix"),
    "gl3_split_mo_ir": dict(N=3, NodeType="gauss-lobatto", SplitDG="mo", Riemann="ir"),
    "gauss5_split_ch_ch": dict(N=5, NodeType="gauss", SplitDG="ch", Riemann="ch"),
    "gauss3_split_ir_lf_br2": dict(N=3, NodeType="gauss", SplitDG="ir", Riemann="lf", Lifting="br2"),
    "gauss4_split_du_roel2": dict(N=4, NodeType="gauss", SplitDG="du", Riemann="roel2"),
    "gauss6_split_mo_gshock": dict(N=6, NodeType="gauss", SplitDG="mo", Riemann="roeentropygshockfix"),
    "gauss3_weak_roel2": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roel2"),
    "gauss3_weak_hll": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hll"),
    "gauss5_weak_hlle_br2": dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="hlle", Lifting="br2"),
    "gauss3_weak_hllem": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="hllem"),
    "gl3_weak_gshock": dict(N=3, NodeType="gauss-lobatto", SplitDG="weak", Riemann="roeentropygshockfix"),
    "gauss9_weak_hllem": dict(N=9, NodeType="gauss", SplitDG="weak", Riemann="hllem"),
}
COMMON = dict(kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.9, DFLScale=0.9)
HALF_DT = {"gl7_split_ch_ch_br2": 0.5, "gl7_split_ir_ir": 0.5}


@pytest.mark.parametrize("name", list(RHS_CASES))
def test_rhs_parity_tgv(name):
    c = product_cfg(**RHS_CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= UT_TOL, err


@pytest.mark.parametrize("name", ["c1_gauss3_weak_roe_br1", "gl7_split_pi_roeef_br2", "gauss5_weak_roeef", "gauss5_split_pi_roeef_br1",
                                  "gauss3_split_sd_lf", "gl5_split_pi_roeef_br2", "gauss11_weak_roeef_br1", "gl11_split_pi_roeef_br2",
                                  "gl7_split_ch_ch_br2", "gauss5_split_ch_ch", "gl7_split_mo_roe", "gauss3_weak_hllem"])
def test_rhs_parity_curved(name):
    c = product_cfg(**RHS_CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3, ngeo=3, perturb=0.2, seed=3)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= UT_TOL, err


@pytest.mark.parametrize("variant", ["split_pi_roe_br1", "split_pi_roeef_br2", "gauss3_weak_lf_br1", "gauss5_split_pi_roeef_br2"])
def test_rhs_parity_channel_walls(variant):
    kw = {"split_pi_roe_br1": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1"),
          "gauss5_split_pi_roeef_br2": dict(N=5, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"),
          "split_pi_roeef_br2": dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2", etaBR2_wall=1.5),
          "gauss3_weak_lf_br1": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="lf", Lifting="br1")}[variant]
    c = product_cfg(**kw, kappa=1.4, R=1.0, Pr=0.72, mu0=1.0 / 2800.0, doTCSource=1, dpdx=-1.0)
    f, o, _ = channel_pair(c, nelems=(3, 4, 2))
    ut_f = f.DGTimeDerivative_weakForm(0.0)
    o.bulk_velocity()  # CalcForcing on the same state
    err = rel_err(ut_f, o.time_derivative(0.0))
    f.close()
    assert err <= UT_TOL, err


@pytest.mark.parametrize("name", ["c1_gauss3_weak_roe_br1", "gl7_split_pi_roeef_br1", "gauss3_weak_br2", "gauss5_split_pi_roeef_br1",
                                  "gauss11_weak_roeef_br1", "gl7_split_ch_ch_br2", "gl7_split_ir_ir", "gauss5_split_ch_ch", "gauss3_weak_hllem",
                                  "gl5_split_kg_avg"])
def test_lserk_steps_fixed_dt(name):
    c = product_cfg(**RHS_CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3)
    dt, err = o.calc_timestep()
    assert err == 0
    # the CH dissipation (like LF's) and the IR volume flux leave the N=7 split operator unstable at CFLScale 0.9 on this
    # noisy state within two steps, on the oracle as on the GPU; half the time step keeps ten steps finite
    dt *= HALF_DT.get(name, 1.0)
    tf = to = 0.0
    for _ in range(10):
        tf = f.TimeStepByLSERKW2(tf, dt)
        to = o.timestep(to, dt)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert abs(tf - to) < 1e-14 and e <= STATE_TOL, e


@pytest.mark.parametrize("name", ["c1_gauss3_weak_roe_br1", "gl7_split_pi_roeef_br2", "gauss11_weak_roeef_br1"])
def test_timedisc_dt_control(name):
    c = product_cfg(**RHS_CASES[name], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3)
    dtf, errf = f.CalcTimeStep()
    dto, erro = o.calc_timestep()
    assert errf == 0 and erro == 0 and abs(dtf - dto) <= 1e-13 * dto
    t = f.TimeDisc(10)
    to = 0.0
    for _ in range(10):
        dt, _ = o.calc_timestep()
        to = o.timestep(to, dt)
    e = rel_err(f.U, o.get_state())
    f.close()
    assert abs(t[0] - to) <= 1e-12 * to and e <= STATE_TOL, (t[0], to, e)


def test_dropin_set_mesh_from_oracle_arrays():
    """fg_set_mesh with the arrays FLEXI's InitMesh would hand over (here: the oracle's)."""
    c = product_cfg(**RHS_CASES["gl7_split_pi_roeef_br2"], **COMMON)
    m = fmesh.tgv_box(3, ngeo=2, perturb=0.2, seed=5)
    o = orc.Oracle(__import__("_cases").oracle_cfg(c), m)
    f = Flexi(c)
    f.set_mesh(o.mesh_iarray("SideToElem"), o.mesh_iarray("ElemToSide"), o.mesh_iarray("BC"), m.boundary_type, m.ref_state_prim,
               o.mesh_array("Mf"), o.mesh_array("Mg"), o.mesh_array("Mh"), o.mesh_array("sJ"), o.mesh_array("NormVec"),
               o.mesh_array("TangVec1"), o.mesh_array("TangVec2"), o.mesh_array("SurfElem"))
    U0 = __import__("_cases").perturb_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), kappa=c.kappa, R=c.R), seed=4)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= UT_TOL, err


def test_freestream_preservation_curved():
    c = product_cfg(**RHS_CASES["gl7_split_pi_roeef_br2"], **COMMON)
    m = fmesh.tgv_box(3, ngeo=7, perturb=0.2, seed=7)
    f = Flexi(c, m)
    U = np.zeros(f.ushape)
    U[..., 0] = 1.2
    U[..., 1] = 1.2 * 0.3
    U[..., 2] = -1.2 * 0.2
    U[..., 3] = 1.2 * 0.1
    U[..., 4] = 100.0 / 0.4 + 0.5 * 1.2 * (0.09 + 0.04 + 0.01)
    f.U = U
    ut = f.DGTimeDerivative_weakForm(0.0)
    f.close()
    assert np.abs(ut).max() < 1e-10 * 250.0, np.abs(ut).max()


def test_conservation_periodic():
    c = product_cfg(**RHS_CASES["c1_gauss3_weak_roe_br1"], **COMMON)
    f, o, _ = tgv_pair(c, n_elem=3, ngeo=2, perturb=0.2)
    ut = f.DGTimeDerivative_weakForm(0.0)
    w = o.mesh_array("wGPVol")
    J = 1.0 / o.mesh_array("sJ")
    tot = np.einsum("eijkv,eijk,ijk->v", ut, J, w)
    scale = np.einsum("eijkv,eijk,ijk->v", np.abs(ut), J, w)
    f.close()
    assert (np.abs(tot) <= 1e-12 * np.maximum(scale, 1.0)).all(), tot


def test_ensemble_matches_separate_instances():
    c = product_cfg(**RHS_CASES["gauss5_weak_roeef"], **COMMON)
    meshes = [fmesh.tgv_box(2), fmesh.tgv_box(3), fmesh.tgv_box(2)]
    machs = [0.1, 0.2, 0.3]
    mus = [1 / 400.0, 1 / 1600.0, 1 / 3200.0]
    ens = fmesh.concatenate(meshes)
    f = Flexi(c, ens)
    f.set_instance_mu0(mus)
    x = f.elem_xgp()
    U0 = np.concatenate([testcases.tgv_state(x[ens.elem_inst == i], mach=machs[i], kappa=c.kappa, R=c.R) for i in range(3)])
    f.U = U0
    t = f.TimeDisc(5)
    Uf = f.U
    f.close()
    off = 0
    for i, m in enumerate(meshes):
        oc = __import__("_cases").oracle_cfg(c)
        oc["mu0"] = mus[i]
        o = orc.Oracle(oc, m)
        o.set_state(U0[off:off + m.n_elems])
        to = 0.0
        for _ in range(5):
            dt, _ = o.calc_timestep()
            to = o.timestep(to, dt)
        assert abs(t[i] - to) <= 1e-12 * to
        assert rel_err(Uf[off:off + m.n_elems], o.get_state()) <= STATE_TOL
        off += m.n_elems


# 0-based row NormalDir of each local side 1..6 (mesh_vars.f90:105-111)
_NORMAL_DIR = {1: 2, 2: 1, 3: 0, 4: 1, 5: 0, 6: 2}


@pytest.mark.parametrize("face_metrics", [False, True])
def test_dropin_gauss_split_face_metrics(face_metrics):
    """Drop-in path for the split form on Gauss nodes: fg_set_mesh alone (face metrics evaluated from the
    volume metrics) and with FLEXI's Ja_Face / Ja_slave handed over by fg_set_face_metrics (here the
    oracle's; the rows other than NormalDir are NaN, so reading one would show)."""
    c = product_cfg(**RHS_CASES["gauss5_split_pi_roeef_br1"], **COMMON)
    m = fmesh.tgv_box(3, ngeo=3, perturb=0.2, seed=6)
    o = orc.Oracle(__import__("_cases").oracle_cfg(c), m)
    f = Flexi(c)
    s2e = o.mesh_iarray("SideToElem")
    f.set_mesh(s2e, o.mesh_iarray("ElemToSide"), o.mesh_iarray("BC"), m.boundary_type, m.ref_state_prim,
               o.mesh_array("Mf"), o.mesh_array("Mg"), o.mesh_array("Mh"), o.mesh_array("sJ"), o.mesh_array("NormVec"),
               o.mesh_array("TangVec1"), o.mesh_array("TangVec2"), o.mesh_array("SurfElem"))
    if face_metrics:
        jm, js = o.mesh_array("JaN_master"), o.mesh_array("JaN_slave")
        n_s, n = jm.shape[0], jm.shape[1]
        JaF = np.full((n_s, n, n, 3, 3), np.nan)
        JaS = np.full((n_s, n, n, 3, 3), np.nan)
        for s_ in range(n_s):
            JaF[s_, :, :, :, _NORMAL_DIR[int(s2e[s_, 2])]] = jm[s_]
            if s2e[s_, 1] > 0:
                JaS[s_, :, :, :, _NORMAL_DIR[int(s2e[s_, 3])]] = js[s_]
        f.set_face_metrics(JaF, JaS)
    U0 = __import__("_cases").perturb_state(testcases.tgv_state(o.mesh_array("Elem_xGP"), kappa=c.kappa, R=c.R), seed=8)
    f.U = U0
    o.set_state(U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= UT_TOL, err
