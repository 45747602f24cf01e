"""Mortar interfaces (mortar.f90, mesh_readin.f90 MortarType/MortarInfo, metrics.f90 Mortar_CalcSurfMetrics)
in the oracle, on the reference's own mortar meshes (tests/golden/hopr/) and its own acceptance criteria.

- cartbox3D_mortar_mesh.h5 (run_basic/freestream_3D, mortar types 1 and 2), Dirichlet sides replaced by
  adiabatic walls: a fluid at rest stays at rest to round-off; the reference's free-stream check on this
  mesh asks for an L2 error below 1e-12.
- periodic mortar meshes (convtest/p_3D_mortar types 1, 2, 3; convtest/h_3D_mortar type 3, flipped sides): a
  constant moving state is preserved and the volume integral of J Ut vanishes for a perturbed state
  (the mortar projection conserves mass, momentum and energy), Gauss weak form, Gauss-Lobatto split form and
  the Gauss split form (entropy-variable prolongation, split-Gauss surface integral), BR1 and BR2 lifting.
- convtest/h_3D_mortar: N=3, IniExactFunc 4 with its source, AdvVel (0.3, 0.3, 0.3), Riemann 33, mu0 1e-3,
  CFLscale = DFLscale = 0.9, tend 1 with the Carpenter RK4-5 scheme on FLIPPED_001, _002, _004: L2 errors below 0.5
  and the mean order of convergence within 15% of N+1 = 4 for at least 80% of the variables
  (analyze_Convtest_h_tolerance 0.15, analyze_Convtest_h_rate 0.8; the reference also runs _008).
- convtest/p_3D_mortar: MORTAR_002, AdvVel (0.3, 0, 0), N = 1..6: L2 errors below 5 and falling with every
  increment of N (the reference runs N = 1..10 and asks for a p-rate of 0.6 on 75% of the increments).
"""
import os

import numpy as np
import pytest

from _cases import l2_error, perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from oracle import oracle as orc

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
BASE = dict(riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, etaBR2=2.0, etaBR2_wall=-1.0, kappa=1.4, R=287.058,
            Pr=0.72, mu0=1e-3, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0)
FORMS = {"gauss-weak": dict(nodeType=orc.NT_GAUSS, splitDG=-1, riemann=33),
         "gl-split-pi": dict(nodeType=orc.NT_GL, splitDG=2, riemann=33),
         "gauss-weak-br2": dict(nodeType=orc.NT_GAUSS, splitDG=-1, riemann=3, lifting=2),
         "gl-split-br2": dict(nodeType=orc.NT_GL, splitDG=2, riemann=33, lifting=2),
         "gauss-split-pi": dict(nodeType=orc.NT_GAUSS, splitDG=4, riemann=33)}
PERIODIC = ["CART_HEX_PERIODIC_MORTAR_002_mesh.h5", "CART_HEX_PERIODIC_MORTAR_FLIPPED_002_mesh.h5"]


def _mesh(name, **kw):
    return fmesh.read_hopr(os.path.join(HOPR, name), **kw)


def test_mortar_tables():
    m = _mesh("CART_HEX_PERIODIC_MORTAR_002_mesh.h5")
    assert m.n_elems == 28 and len(m.mortars) == 8 and sorted(set(m.mortars[:, 2].tolist())) == [1, 2, 3]
    f = _mesh("CART_HEX_PERIODIC_MORTAR_FLIPPED_002_mesh.h5")
    assert f.n_elems == 12 and len(f.mortars) == 8 and (f.mortars[:, 2] == 3).all()
    for mm in (m, f):
        for row in mm.mortars:
            big, ls, typ = row[:3]
            assert mm.elem_nb[big - 1, ls - 1, 0] == -1  # the big side is a mortar side
            for k in range(4 if typ == 1 else 2):
                se, sls, flip = row[3 + 3 * k: 6 + 3 * k]
                assert mm.elem_nb[se - 1, sls - 1, 0] == -1 and flip == 0
        # every side with neighbour -1 is a big or small mortar side
        n_small = sum(4 if r[2] == 1 else 2 for r in mm.mortars)
        assert (mm.elem_nb[:, :, 0] == -1).sum() == len(mm.mortars) + n_small
    c = _mesh("cartbox3D_mortar_mesh.h5")
    assert sorted(set(c.mortars[:, 2].tolist())) == [1, 2]


def test_fluid_at_rest_on_mortar_box():
    m0 = _mesh("cartbox3D_mortar_mesh.h5")
    m = _mesh("cartbox3D_mortar_mesh.h5", boundary={nm: (3, 0) for nm in m0.bc_names if nm != "inner"})
    for form in FORMS.values():
        o = orc.Oracle(dict(BASE, N=3, **form), m)
        x = o.mesh_array("Elem_xGP")
        U = np.zeros(x.shape[:-1] + (5,))
        U[..., 0] = 1.0
        U[..., 4] = 1.0 / 0.4
        o.set_state(U)
        assert np.abs(o.time_derivative(0.0)).max() <= 1e-12


@pytest.mark.parametrize("name", PERIODIC)
@pytest.mark.parametrize("form", list(FORMS))
def test_free_stream_and_conservation(name, form):
    m = _mesh(name)
    o = orc.Oracle(dict(BASE, N=4, **FORMS[form]), m)
    x = o.mesh_array("Elem_xGP")
    U = np.empty(x.shape[:-1] + (5,))
    U[...] = [1.2, 0.3, -0.2, 0.5, 3.1]
    o.set_state(U)
    assert np.abs(o.time_derivative(0.0)).max() <= 1e-12
    U = perturb_state(testcases.sine_wave_state(x, 0.0, (0.3, 0.3, 0.3)), seed=3, amp=0.1)
    o.set_state(U)
    Ut = o.time_derivative(0.0)
    w = orc.nodes_and_weights(4, FORMS[form]["nodeType"])[1]
    W = np.einsum('a,b,c->abc', w, w, w) / o.mesh_array("sJ")
    total = (Ut * W[..., None]).sum(axis=(0, 1, 2, 3))
    scale = (np.abs(Ut) * W[..., None]).sum(axis=(0, 1, 2, 3))
    assert (np.abs(total) <= 1e-13 * scale).all(), (total, scale)


@pytest.mark.parametrize("perturb", [0.0, 0.1])
@pytest.mark.parametrize("form", list(FORMS))
def test_synthetic_mortar_box(perturb, form):
    """The library's periodic mortar box (flexi_gb300.mesh.mortar_box, both zeta faces of every coarse element
    1->4 mortars, the small sides on both orientations of the big side): free stream and conservation."""
    m = fmesh.mortar_box(4, perturb=perturb, seed=2)
    assert m.n_elems == 160 and len(m.mortars) == 64
    o = orc.Oracle(dict(BASE, N=4, **FORMS[form]), m)
    x = o.mesh_array("Elem_xGP")
    U = np.empty(x.shape[:-1] + (5,))
    U[...] = [1.2, 0.3, -0.2, 0.5, 3.1]
    o.set_state(U)
    assert np.abs(o.time_derivative(0.0)).max() <= 2e-12
    o.set_state(perturb_state(testcases.sine_wave_state(x, 0.0, (0.3, 0.3, 0.3)), seed=3, amp=0.1))
    Ut = o.time_derivative(0.0)
    w = orc.nodes_and_weights(4, FORMS[form]["nodeType"])[1]
    W = np.einsum('a,b,c->abc', w, w, w) / o.mesh_array("sJ")
    total = (Ut * W[..., None]).sum(axis=(0, 1, 2, 3))
    scale = (np.abs(Ut) * W[..., None]).sum(axis=(0, 1, 2, 3))
    assert (np.abs(total) <= 1e-13 * scale).all(), (total, scale)


def _sine_wave_run(name, N, adv, t_end=1.0):
    cfg = dict(BASE, N=N, iniExactFunc=4, advVel=adv, **FORMS["gauss-weak"])
    o = orc.Oracle(cfg, _mesh(name))
    x = o.mesh_array("Elem_xGP")
    o.set_state(testcases.sine_wave_state(x, 0.0, adv))
    t = 0.0
    while t < t_end - 1e-12:
        dt, err = o.calc_timestep()
        assert err == 0
        t = o.timestep(t, min(dt, t_end - t))
    return l2_error(N, orc.NT_GAUSS, x, o.mesh_array("sJ"), o.get_state(),
                    lambda xa: testcases.sine_wave_state(xa, t_end, adv))


def test_h_convergence_mortar():
    orc.set_threads(orc.max_threads())
    errs = np.array([_sine_wave_run(f"CART_HEX_PERIODIC_MORTAR_FLIPPED_{k:03d}_mesh.h5", 3, (0.3, 0.3, 0.3)) for k in (1, 2, 4)])
    assert (errs < 0.5).all()
    order = np.log2(errs[:-1] / errs[1:]).mean(axis=0)
    ok = np.abs(order / 4.0 - 1.0) <= 0.15
    assert ok.mean() >= 0.8, order


def test_p_convergence_mortar():
    orc.set_threads(orc.max_threads())
    errs = np.array([_sine_wave_run("CART_HEX_PERIODIC_MORTAR_002_mesh.h5", N, (0.3, 0.0, 0.0)) for N in range(1, 7)])
    assert (errs < 5.0).all()
    assert (errs[1:] < errs[:-1]).all(), errs
