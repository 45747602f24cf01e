"""Wall-bounded adjoint: channel with isothermal walls, channel body force and a body-force field.

Bars: the forward with a body-force field matches the oracle (Ut within 1e-12, as every forward parity
test); the gradients of a linear functional of the state after a fixed-dt solve with respect to the
initial state, the viscosity multipliers and the body-force field pass the dot-product test against the
oracle's exact (dual-number) tangent of the solve, bulk-velocity coupling included, within 1e-10 of the
sum of |JV_i w_i|; the mean wall shear of a laminar Poiseuille state on straight elements is 3 mu to
round-off (1e-10); its gradient on the stretched channel matches a Richardson-extrapolated central
difference within 1e-8 (the wall shear involves no Riemann solver, so it has no kinks)."""
import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

N_STEPS = 5


def _channel(seed=0, with_field=True, **kw):
    cfg = dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1", mu0=5e-3, R=1.0, doTCSource=1, dpdx=-0.5,
               CFLScale=0.5, DFLScale=0.5)
    cfg.update(kw)
    c = make_config(**cfg)
    m = fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2, t_wall=1.0)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = perturb_state(testcases.channel_state(f.elem_xgp(), mach=0.3, kappa=c.kappa, R=c.R, t_wall=1.0, noise=0.0, seed=seed),
                       seed=seed + 9, amp=0.03)
    rng = np.random.default_rng(seed + 77)
    F = 0.2 * rng.standard_normal(f.ushape[:-1]) if with_field else None
    scale = rng.uniform(0.8, 1.2, f.n_elems)
    f.U = U0
    f.set_elem_mu_scale(scale)
    o.set_state(U0)
    o.set_mu_scale(scale)
    if F is not None:
        f.set_body_force_field(F)
        o.set_force_field(F)
    return f, o, U0, F, scale, rng


def test_forward_with_body_force_field():
    f, o, U0, F, scale, rng = _channel()
    o.bulk_velocity()  # bulk velocity of this state on the oracle side (the GPU computes its own)
    assert rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative()) <= 1e-12
    # one RK step: both sides take the bulk velocity of the step start
    dt = 1e-3
    f.TimeStepByLSERKW2(0.0, dt)
    o.set_state(U0)
    o.timestep(0.0, dt)
    assert rel_err(f.U, o.get_state()) <= 1e-10


def test_solve_adjoint_with_body_force_against_exact_tangent():
    f, o, U0, F, scale, rng = _channel(seed=1)
    dt = float(np.atleast_1d(f.CalcTimeStep()[0])[0])
    f.U = U0
    f.adjoint_forward(N_STEPS, dt, 2)
    w = rng.standard_normal(f.ushape)
    Ub0, mub, fb = f.adjoint_reverse(w, force_bar=True)
    V = rng.standard_normal(f.ushape) * np.abs(U0).max(axis=(0, 1, 2, 3))
    ds = rng.standard_normal(f.n_elems)
    dF = rng.standard_normal(f.ushape[:-1])
    for name, tang, got in (("state", o.jvp_solve(V, N_STEPS, dt), float((Ub0 * V).sum())),
                            ("viscosity", o.jvp_solve(None, N_STEPS, dt, d_scale=ds), float(mub @ ds)),
                            ("body force", o.jvp_solve(None, N_STEPS, dt, d_force=dF), float((fb * dF).sum()))):
        lhs = float((tang * w).sum())
        assert abs(lhs - got) <= 1e-10 * float(np.abs(tang * w).sum()), (name, lhs, got)


def test_wall_shear_value_and_gradient():
    # on straight elements the Poiseuille parabola u = 1.5 (1 - y^2) is a polynomial of degree 2 < N, so the
    # lifted wall gradient and the mean wall shear 3 mu are exact
    c = make_config(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br1", mu0=5e-3, R=1.0)
    m = fmesh.cartesian_box((2, 3, 2), (0.0, -1.0, 0.0), (2 * np.pi, 1.0, np.pi), ngeo=1, periodic=(True, False, True), wall_bc=(4, 1),
                            ref_state_prim=np.array([[1.0, 0.0, 0.0, 0.0, 1.0, 1.0]]))
    fc = Flexi(c, m)
    fc.U = testcases.channel_state(fc.elem_xgp(), mach=0.1, kappa=1.4, R=1.0, t_wall=1.0, noise=0.0, seed=0)
    assert abs(fc.wall_shear() - 3 * 5e-3) <= 1e-10 * 3 * 5e-3
    f, o, U0, F, scale, rng = _channel(seed=2, with_field=False, doTCSource=0)
    f.U = U0
    J0, g = f.wall_shear(grad=True)
    V = rng.standard_normal(f.ushape) * np.abs(U0).max(axis=(0, 1, 2, 3))

    def Jof(U):
        f.U = U
        return f.wall_shear()

    h = 1e-4  # fourth-order Richardson quotient: truncation ~h^4, round-off / h ~1e-11
    d1 = (Jof(U0 + h * V) - Jof(U0 - h * V)) / (2 * h)
    d2 = (Jof(U0 + 2 * h * V) - Jof(U0 - 2 * h * V)) / (4 * h)
    rich = (4 * d1 - d2) / 3
    assert abs(float((g * V).sum()) - rich) <= 1e-8 * abs(rich), (float((g * V).sum()), rich)
