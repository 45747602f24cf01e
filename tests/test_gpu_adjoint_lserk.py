"""Adjoint of the LSERK time stepper (fg_adjoint_forward / fg_adjoint_reverse) and its autograd binding.

Bars: the gradients with respect to the initial state and the viscosity multipliers pass the dot-product
test against the oracle's exact (dual-number) tangent of the whole solve within 1e-10 of the sum of
|JV_i w_i|; for the 5-stage RoeEntropyFix cases both also agree with central differences of the same fixed-dt
solve: the state gradient within 1e-8 (h = 1e-6), the multiplier gradient within 3e-8 (h = 1e-3). Step sizes and
bars come from h-sweeps of these functionals against the adjoint: the state quotient is accurate to 3e-10..1.5e-9
at h = 1e-6 and straddles the entropy fix's branch points at some of the ~10^4 face-point evaluations from
h = 2e-6..1e-5 on (Richardson extrapolation from h and 2h then fails by 1e-7); the multiplier derivatives are
1e-4 of the functional, and their quotients reach a round-off floor of 0.5..1.7e-8 at h = 1e-3 (error ~1/h below,
~h^2 and branch crossings above). The exact tangent is the primary check. The result does not depend on the
checkpoint interval (identical to round-off, 1e-13); a kinetic-energy loss differentiated through
flexi_gb300.autograd matches its Richardson-extrapolated finite difference within 1e-8. The other cases are held to the exact
tangent only: the plain Roe flux has a kink at a zero eigenvalue and HLLC wave-speed branches, which a
finite difference can straddle somewhere among a thousand face points and 35 stages; the 14-stage scheme's
3.4x larger steps and the overintegration case made the central differences drift by 2e-5 and 6e-6 while
their dot-product tests held at 1e-10. The reverse sweep runs every low-storage scheme (3, 5 and 14 stages
here) and the transposed overintegration filter."""
import numpy as np
import pytest
import torch

from _cases import oracle_cfg, perturb_state
from flexi_gb300 import autograd as fgad, mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

CASES = {
    "gauss3_weak_roeef_br1": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1"),
    "gl3_split_pi_roe_br2": dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br2"),
    # the other low-storage schemes (TimeDiscMethod): Niegemann RK4-14 and the standard RK3-3
    "gauss3_weak_roeef_br1_niegemann14": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1",
                                              TimeDiscMethod=2),
    "gl3_split_pi_roeef_br1_rk33": dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1",
                                        TimeDiscMethod=1),
    # the discretisation of the N=7 TGV benchmark (split PI, HLLC, BR2) at N=3
    "gl3_split_pi_hllc_br2": dict(N=3, NodeType="gauss-lobatto", SplitDG="pi", Riemann="hllc", Lifting="br2"),
    # split form on Gauss nodes (the discretisation of the reference's tgv/splitGauss regression at N=3)
    "gauss3_split_pi_roeef_br1": dict(N=3, NodeType="gauss", SplitDG="pi", Riemann="roeentropyfix", Lifting="br1"),
    # overintegration: the stage right-hand sides carry the cut-off filter, the reverse sweep its transpose
    "gauss3_weak_roe_br1_cutoff": dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1",
                                       OverintegrationType=1, NUnder=2),
}
N_STEPS = 7


def _setup(name, seed=0):
    c = make_config(mu0=5e-3, R=71.42857, CFLScale=0.5, DFLScale=0.5, **CASES[name])
    m = fmesh.tgv_box(3, ngeo=2, perturb=0.05, seed=seed)
    f = Flexi(c, m)
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.3, kappa=c.kappa, R=c.R), seed=seed + 3, amp=0.05)
    rng = np.random.default_rng(seed + 50)
    scale = rng.uniform(0.8, 1.2, f.n_elems)
    f.U = U0
    f.set_elem_mu_scale(scale)
    dt, _ = f.CalcTimeStep()
    return f, U0, scale, float(np.atleast_1d(dt)[0]), rng


def _solve(f, U0, scale, dt, every=N_STEPS):
    f.U = U0
    f.set_elem_mu_scale(scale)
    f.adjoint_forward(N_STEPS, dt, every)
    return f.U


def _central(J, x, dx, h):
    return (J(x + h * dx) - J(x - h * dx)) / (2 * h)


def _rich(J, x, dx, h):
    d1 = (J(x + h * dx) - J(x - h * dx)) / (2 * h)
    d2 = (J(x + 2 * h * dx) - J(x - 2 * h * dx)) / (4 * h)
    return (4 * d1 - d2) / 3


@pytest.mark.parametrize("name", list(CASES))
def test_lserk_adjoint_against_exact_tangent_and_finite_differences(name):
    f, U0, scale, dt, rng = _setup(name)
    w = rng.standard_normal(U0.shape)
    _solve(f, U0, scale, dt, every=3)
    Ub0, mub = f.adjoint_reverse(w)
    V = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
    o = orc.Oracle(oracle_cfg(f.cfg), fmesh.tgv_box(3, ngeo=2, perturb=0.05, seed=0))
    o.set_state(U0)
    o.set_mu_scale(scale)
    JV = o.jvp_solve(V, N_STEPS, dt)
    lhs, rhs = float((JV * w).sum()), float((Ub0 * V).sum())
    assert abs(lhs - rhs) <= 1e-10 * float(np.abs(JV * w).sum()), (lhs, rhs)
    if CASES[name]["Riemann"] not in ("roe", "hllc"):
        fdU = _central(lambda U: float((_solve(f, U, scale, dt) * w).sum()), U0, V, 1e-6)
        assert abs(rhs - fdU) <= 1e-8 * abs(fdU), (rhs, fdU)
    ds = rng.standard_normal(f.n_elems)
    Js = o.jvp_solve(None, N_STEPS, dt, d_scale=ds)
    lhs = float((Js * w).sum())
    assert abs(lhs - float(mub @ ds)) <= 1e-10 * float(np.abs(Js * w).sum()), (lhs, float(mub @ ds))
    if CASES[name]["Riemann"] not in ("roe", "hllc"):
        # the viscosity sensitivity is small next to the functional: a larger step keeps round-off out of the quotient
        fds = _central(lambda s: float((_solve(f, U0, s, dt) * w).sum()), scale, ds, 1e-3)
        assert abs(float(mub @ ds) - fds) <= 3e-8 * abs(fds), (float(mub @ ds), fds)


@pytest.mark.parametrize("recompute", ["0", "1"])
def test_checkpoint_interval_does_not_change_the_gradient(recompute, monkeypatch):
    """Both reverse paths (kept stage intermediates / recomputed ones) and every checkpoint interval give
    the same gradient."""
    monkeypatch.setenv("FLEXI_GB300_ADJOINT_RECOMPUTE", recompute)
    f, U0, scale, dt, rng = _setup("gauss3_weak_roeef_br1", seed=4)
    w = rng.standard_normal(U0.shape)
    ref = None
    for every in (1, 3, N_STEPS):
        UT = _solve(f, U0, scale, dt, every=every)
        Ub0, mub = f.adjoint_reverse(w)
        assert np.array_equal(f.U, UT)  # the state is left at t_end
        if ref is None:
            ref = (Ub0, mub)
        else:
            assert np.abs(Ub0 - ref[0]).max() <= 1e-13 * np.abs(ref[0]).max()
            assert np.abs(mub - ref[1]).max() <= 1e-13 * np.abs(ref[1]).max()


def test_autograd_kinetic_energy_loss():
    f, U0, scale, dt, rng = _setup("gauss3_weak_roeef_br1", seed=5)
    n = f.n
    _, w1, _ = orc.nodes_and_weights(f.N, 1)
    w3 = torch.from_numpy(np.einsum("k,j,i->kji", w1, w1, w1))
    jac = torch.from_numpy(1.0 / f.mesh_array("sJ"))
    target = 0.5

    def loss_of(U0_t, s_t):
        UT = fgad.Solve.apply(U0_t, s_t, f, N_STEPS, dt, 3)
        return (fgad.kinetic_energy(UT, w3, jac) - target) ** 2

    U0_t = torch.from_numpy(U0.copy()).requires_grad_(True)
    s_t = torch.from_numpy(scale.copy()).requires_grad_(True)
    loss = loss_of(U0_t, s_t)
    loss.backward()
    V = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
    ds = rng.standard_normal(f.n_elems)

    def L(U, s):
        with torch.no_grad():
            return float(loss_of(torch.from_numpy(U), torch.from_numpy(s)))

    fdU = _rich(lambda U: L(U, scale), U0, V, 1e-6)
    fds = _rich(lambda s: L(U0, s), scale, ds, 1e-3)
    assert abs(float((U0_t.grad.numpy() * V).sum()) - fdU) <= 1e-8 * abs(fdU)
    assert abs(float(s_t.grad.numpy() @ ds) - fds) <= 1e-8 * abs(fds)


def _binomial_recomputations(n, nsnap):
    """Forward steps the binomial schedule of fg_adjoint_reverse re-runs (a model of the same rule:
    snapshot so that the part after it is the longest reversible with one slot less, at the smallest
    sufficient repetition count; the forward pass stores the first right spine)."""
    from math import comb

    def split(t, s):
        r = 0
        while comb(s + r, s) < t:
            r += 1
        return t - min(t - 1, comb(s - 1 + r, s - 1))

    spine, l, s = set(), 0, nsnap - 1
    while n - l > 1 and s > 0:
        l += split(n - l, s)
        spine.add(l)
        s -= 1
    count = 0

    def rev(l, r, s):
        nonlocal count
        if r - l == 1:
            count += 1
            return
        if s == 0:
            count += sum(i - l + 1 for i in range(l, r))
            return
        m = l + split(r - l, s)
        if m in spine:
            spine.discard(m)
        else:
            count += m - l
        rev(m, r, s - 1)
        rev(l, m, s)

    rev(0, n, nsnap - 1)
    return count


def test_binomial_checkpointing_matches_uniform():
    """Binomial (revolve) schedules with 1..n+1 snapshots give the gradient of uniform checkpointing, leave
    the state at t_end, and re-run exactly the forward steps of the schedule (n(n+1)/2 with one snapshot,
    n with n snapshots or more); a second reverse sweep needs a new forward."""
    f, U0, scale, dt, rng = _setup("gauss3_weak_roeef_br1", seed=6)
    n = 13
    w = rng.standard_normal(U0.shape)
    f.U = U0
    f.adjoint_forward(n, dt, ckpt_every=n)
    UT = f.U
    ref, mref = f.adjoint_reverse(w)
    assert f.adjoint_recomputed_steps() == n
    for nsnap in (1, 2, 3, 5, n + 1):
        f.U = U0
        f.adjoint_forward(n, dt, snapshots=nsnap)
        assert np.array_equal(f.U, UT)
        Ub0, mub = f.adjoint_reverse(w)
        assert np.array_equal(f.U, UT)
        assert np.abs(Ub0 - ref).max() <= 1e-13 * np.abs(ref).max(), nsnap
        assert np.abs(mub - mref).max() <= 1e-13 * np.abs(mref).max(), nsnap
        assert f.adjoint_recomputed_steps() == _binomial_recomputations(n, nsnap), nsnap
        with pytest.raises(Exception):
            f.adjoint_reverse(w)
    assert _binomial_recomputations(n, 1) == n * (n + 1) // 2
    assert _binomial_recomputations(n, n + 1) == n


def test_lserk_adjoint_with_time_dependent_source():
    """Exact function 4 with its source (stage times t + RKc dt): the reverse sweep recomputes its steps at
    the times of the forward solve (started at fg_set_time's t = 0, as the oracle's tangent solve starts);
    the dot-product test against the oracle's exact tangent of the solve holds at 1e-10."""
    adv = (0.3, 0.3, 0.3)
    c = make_config(N=3, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix", Lifting="br1", mu0=5e-3, R=287.058,
                    CFLScale=0.5, DFLScale=0.5, IniExactFunc=4, AdvVel=adv)
    m = fmesh.cartesian_box((3, 3, 3), (-1.0,) * 3, (1.0,) * 3)
    f = Flexi(c, m)
    U0 = perturb_state(testcases.sine_wave_state(f.elem_xgp(), 0.0, adv), seed=1, amp=0.05)
    f.U = U0
    dt = float(np.atleast_1d(f.CalcTimeStep()[0])[0])
    rng = np.random.default_rng(9)
    w = rng.standard_normal(U0.shape)
    for every in (3, N_STEPS):
        f.set_time(0.0)
        f.U = U0
        f.adjoint_forward(N_STEPS, dt, every)
        Ub0, _ = f.adjoint_reverse(w)
        V = rng.standard_normal(U0.shape) * np.abs(U0).max(axis=(0, 1, 2, 3))
        o = orc.Oracle(oracle_cfg(f.cfg), m)
        o.set_state(U0)
        JV = o.jvp_solve(V, N_STEPS, dt)
        lhs, rhs = float((JV * w).sum()), float((Ub0 * V).sum())
        assert abs(lhs - rhs) <= 1e-10 * float(np.abs(JV * w).sum()), (every, lhs, rhs)
    f.close()
