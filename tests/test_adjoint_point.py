"""Point-wise adjoints (fg_adjoint_point.cuh) against central finite differences of the same forward code.

Runs on the CPU through libfgpoint.so, the point-wise functions compiled as host code. For random
physical states x, random output cotangents yb and random directions dx, the adjoint gives xb = J^T yb
and the test compares <xb, dx> with <yb, (f(x + h dx) - f(x - h dx)) / 2h>, Richardson-extrapolated
from h and 2h (h = 1e-5; 2e-6 for RoeEntropyGShockFix and the logarithmic means of CH and IR). Samples whose finite
difference straddles a branch of the forward function (entropy fix, max, abs, pressure clamp) are
recognised by two step sizes disagreeing and skipped; the test asserts that most samples are kept."""
import ctypes
import os

import numpy as np
import pytest

from flexi_gb300 import build as fbuild

KAPPA, RGAS = 1.4, 287.058
TOL = 2e-7


@pytest.fixture(scope="module")
def pt():
    path = fbuild.build_point_harness()
    L = ctypes.CDLL(path)
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.fgpt_cons_to_prim.argtypes = [D, D, P, P]
    L.fgpt_cons_to_prim_adj.argtypes = [D, D, P, P, P]
    L.fgpt_visc.argtypes = [D, P, P, P]
    L.fgpt_visc_adj.argtypes = [D, P, P, P, P]
    L.fgpt_visc_phys.argtypes = [D, P, P]
    L.fgpt_visc_phys_adj.argtypes = [D, P, P, P]
    L.fgpt_riemann.argtypes = [I, I, D, D, P, P, P]
    L.fgpt_riemann_adj.argtypes = [I, I, D, D, P, P, P, P, P]
    L.fgpt_split_pair_gen.argtypes = [I, P, P, P]
    L.fgpt_split_pair_gen_adj.argtypes = [I, P, P, P, P]
    L.fgpt_split_node_inputs.argtypes = [I, P, P]
    L.fgpt_split_node_inputs_adj.argtypes = [I, P, P, P]
    L.fgpt_split_surface_more.argtypes = [I, P, P, P]
    L.fgpt_split_surface_more_adj.argtypes = [I, P, P, P, P, P]
    L.fgpt_riemann_more.argtypes = [I, I, D, D, D, P, P, P]
    L.fgpt_riemann_more_adj.argtypes = [I, I, D, D, D, P, P, P, P, P]
    L.fgpt_pressure_riemann.argtypes = [D, D, P]
    L.fgpt_pressure_riemann.restype = D
    L.fgpt_pressure_riemann_adj.argtypes = [D, D, P, D, P]
    L.fgpt_split_pair.argtypes = [I, P, P, P]
    L.fgpt_split_pair_adj.argtypes = [I, P, P, P, P]
    L.fgpt_split_inputs.argtypes = [I, P, P]
    L.fgpt_split_inputs_adj.argtypes = [I, P, P, P]
    for nm in ("fgpt_cons_to_entropy", "fgpt_entropy_to_cons"):
        getattr(L, nm).argtypes = [D, P, P]
        getattr(L, nm + "_adj").argtypes = [D, P, P, P]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(f, fadj, x, nout, rng, n_dirs=3, hs=(1e-5, 2e-5), cancel=0.0):
    """Returns the worst relative mismatch over a few directions, or None if a branch was crossed. cancel > 0 also measures
    the mismatch against cancel * sum_i |xb_i dx_i|, for directions whose derivative is a near-cancelling sum (there the
    quotient's round-off, relative to the small derivative, says nothing about the adjoint)."""
    worst = 0.0
    for _ in range(n_dirs):
        yb = rng.standard_normal(nout)
        dx = rng.standard_normal(x.size) * np.maximum(np.abs(x), 1e-3)
        xb = fadj(x, yb)
        lhs = float(xb @ dx)
        fd = []
        for h in hs:
            fd.append(float(yb @ (f(x + h * dx) - f(x - h * dx)) / (2 * h)))
        rich = (4.0 * fd[0] - fd[1]) / 3.0  # Richardson: O(h^4)
        scale = max(abs(lhs), abs(rich), 1e-8 * (np.abs(xb).sum() * np.abs(dx).max() + 1e-300), cancel * float(np.abs(xb * dx).sum()))
        if abs(fd[0] - fd[1]) > 1e-4 * scale:
            return None
        worst = max(worst, abs(lhs - rich) / scale)
    return worst


def _state(rng, vmax=1.0):
    rho = rng.uniform(0.5, 2.0)
    v = rng.uniform(-vmax, vmax, 3)
    p = rng.uniform(0.5, 3.0)
    E = p / (KAPPA - 1) + 0.5 * rho * (v @ v)
    return np.array([rho, 1.0 / rho, E, p, v[0], v[1], v[2]])


def test_cons_to_prim_adjoint(pt):
    rng = np.random.default_rng(1)

    def f(U):
        out = np.empty(6)
        pt.fgpt_cons_to_prim(KAPPA, RGAS, _p(U), _p(out))
        return np.concatenate([out, [U[0], U[4]]])  # face states also carry rho and E directly

    def fadj(U, yb):
        Ub = np.empty(5)
        pt.fgpt_cons_to_prim_adj(KAPPA, RGAS, _p(U), _p(np.ascontiguousarray(yb)), _p(Ub))
        return Ub

    for _ in range(50):
        s = _state(rng)
        U = np.array([s[0], s[0] * s[4], s[0] * s[5], s[0] * s[6], s[2]])
        err = _check(f, fadj, U, 8, rng)
        assert err is not None and err < TOL, err


def test_viscous_flux_adjoint(pt):
    rng = np.random.default_rng(2)
    lamfac = RGAS * KAPPA / (KAPPA - 1) / 0.72
    for _ in range(50):
        x = np.concatenate([rng.uniform(-1, 1, 3), rng.standard_normal(12), [rng.uniform(1e-4, 1e-2)]])
        m = rng.standard_normal(3)

        def f(x):
            out = np.empty(4)
            pt.fgpt_visc(lamfac, _p(x), _p(m), _p(out))
            return out

        def fadj(x, yb):
            xb = np.empty(16)
            pt.fgpt_visc_adj(lamfac, _p(x), _p(m), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 4, rng)
        assert err is not None and err < TOL, err


def test_physical_viscous_flux_adjoint(pt):
    rng = np.random.default_rng(4)
    lamfac = RGAS * KAPPA / (KAPPA - 1) / 0.72
    for _ in range(50):
        x = np.concatenate([rng.uniform(-1, 1, 3), rng.standard_normal(12), [rng.uniform(1e-4, 1e-2)]])

        def f(x):
            out = np.empty(12)
            pt.fgpt_visc_phys(lamfac, _p(x), _p(out))
            return out

        def fadj(x, yb):
            xb = np.empty(16)
            pt.fgpt_visc_phys_adj(lamfac, _p(x), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 12, rng)
        assert err is not None and err < TOL, err


@pytest.mark.parametrize("solver", [1, 2, 3, 33])
@pytest.mark.parametrize("split", [-1, 4, 0])
def test_riemann_adjoint(pt, solver, split):
    rng = np.random.default_rng(10 * solver + split + 5)
    kept, n = 0, 120
    for it in range(n):
        L, R = _state(rng, vmax=1.6), _state(rng, vmax=1.6)
        x = np.concatenate([L, R])

        def f(x):
            F = np.empty(5)
            pt.fgpt_riemann(solver, split, KAPPA, RGAS, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])), _p(F))
            return F

        def fadj(x, yb):
            Lb, Rb = np.empty(7), np.empty(7)
            pt.fgpt_riemann_adj(solver, split, KAPPA, RGAS, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])),
                                _p(np.ascontiguousarray(yb)), _p(Lb), _p(Rb))
            return np.concatenate([Lb, Rb])

        err = _check(f, fadj, x, 5, rng)
        if err is None:
            continue
        kept += 1
        assert err < TOL, (it, err)
    assert kept >= 0.8 * n


# HLL, HLLE, HLLEM, RoeL2, RoeEntropyGShockFix with the weak form and the split forms PI / SD, the flux average with PI / SD
MORE_CASES = ([(s, sp) for s in (4, 5, 6, 32, 34) for sp in (-1, 4, 0)] + [(0, 4), (0, 0)] +
              # the split fluxes MO (1), DU (2), KG (3): every solver with a central part, and the flux average
              [(s, sp) for s in (1, 2, 3, 33, 32, 34, 0) for sp in (1, 2, 3)] + [(5, 1)] +
              # CH (5) and IR (6): the split forms with every solver with a central part; the CH (7) and IR (8) surface fluxes
              [(s, sp) for s in (1, 3, 33, 32, 34, 0) for sp in (5, 6)] + [(s, sp) for s in (7, 8) for sp in (4, 0, 1, 5, 6)])


@pytest.mark.parametrize("solver,split", MORE_CASES)
def test_riemann_more_adjoint(pt, solver, split):
    rng = np.random.default_rng(100 + 10 * solver + split)
    phi = 5.0  # RiemannPhiFactor of RoeEntropyGShockFix
    kept, n = 0, 120
    for it in range(n):
        L, R = _state(rng, vmax=1.6), _state(rng, vmax=1.6)
        x = np.concatenate([L, R])

        def f(x):
            F = np.empty(5)
            pt.fgpt_riemann_more(solver, split, KAPPA, RGAS, phi, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])), _p(F))
            return F

        def fadj(x, yb):
            Lb, Rb = np.empty(7), np.empty(7)
            pt.fgpt_riemann_more_adj(solver, split, KAPPA, RGAS, phi, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])),
                                     _p(np.ascontiguousarray(yb)), _p(Lb), _p(Rb))
            return np.concatenate([Lb, Rb])

        # smaller steps for RoeEntropyGShockFix and wherever a logarithmic mean enters (CH, IR): next to the entropy-fix
        # branches the flux curves strongly, and the log mean switches between its series and its logarithm at |f| = 0.1 with
        # a slight jump of the derivative; steps of 1e-5 straddle either at some samples (errors up to 3e-6 that vanish at
        # 3e-6). The other cases keep the larger steps, whose round-off is lower.
        # (the smaller steps carry more round-off, which near-cancelling directions of these long flux chains show: their
        # mismatch is also measured against 1e-2 of sum |xb_i dx_i|)
        small = solver in (34, 7, 8) or split in (5, 6)
        err = _check(f, fadj, x, 5, rng, hs=(2e-6, 4e-6) if small else (1e-5, 2e-5), cancel=1e-2 if small else 1e-3)
        if err is None:
            continue
        kept += 1
        assert err < TOL, (it, err)
    assert kept >= 0.8 * n


def test_pressure_riemann_adjoint(pt):
    rng = np.random.default_rng(3)
    kept = 0
    for it in range(100):
        rho, p = rng.uniform(0.5, 2.0), rng.uniform(0.5, 3.0)
        vn = rng.uniform(-1.5, 1.5)
        x = np.array([rho, vn, p])

        def f(x):
            return np.array([pt.fgpt_pressure_riemann(KAPPA, RGAS, _p(np.ascontiguousarray(x)))])

        def fadj(x, yb):
            xb = np.empty(3)
            pt.fgpt_pressure_riemann_adj(KAPPA, RGAS, _p(np.ascontiguousarray(x)), float(yb[0]), _p(xb))
            return xb

        err = _check(f, fadj, x, 1, rng)
        if err is None:
            continue
        kept += 1
        assert err < TOL, (it, err)
    assert kept >= 90


@pytest.mark.parametrize("pi", [1, 0])
def test_split_pair_flux_adjoint(pt, pi):
    """Two-point volume flux of the split form (PI, SD) transposed, w.r.t. both nodes' inputs."""
    rng = np.random.default_rng(20 + pi)
    for _ in range(50):
        x = np.concatenate([rng.uniform(0.5, 2.0, 1), rng.uniform(-1, 1, 3), rng.uniform(0.5, 3.0, 2),
                            rng.uniform(0.5, 2.0, 1), rng.uniform(-1, 1, 3), rng.uniform(0.5, 3.0, 2)])
        ms = rng.standard_normal(3)

        def f(x):
            G = np.empty(5)
            pt.fgpt_split_pair(pi, _p(np.ascontiguousarray(x)), _p(ms), _p(G))
            return G

        def fadj(x, yb):
            xb = np.empty(12)
            pt.fgpt_split_pair_adj(pi, _p(np.ascontiguousarray(x)), _p(ms), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 5, rng)
        assert err is not None and err < TOL, err


@pytest.mark.parametrize("pi", [1, 0])
def test_split_inputs_adjoint(pt, pi):
    rng = np.random.default_rng(30 + pi)
    for _ in range(30):
        s = _state(rng)
        x = np.array([s[0], s[2], s[4], s[5], s[6], s[3], s[1]])  # rho, E, u, v, w, p, 1/rho as independent fields

        def f(x):
            q = np.empty(6)
            pt.fgpt_split_inputs(pi, _p(np.ascontiguousarray(x)), _p(q))
            return q

        def fadj(x, yb):
            xb = np.empty(7)
            pt.fgpt_split_inputs_adj(pi, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 6, rng)
        assert err is not None and err < TOL, err


@pytest.mark.parametrize("sd", [0, 4, 1, 2, 3, 5, 6])
def test_split_pair_flux_gen_adjoint(pt, sd):
    """Two-point volume flux of every split form, transposed, w.r.t. both nodes' inputs (CH: q4 = rho / 2p, IR: q0 = sqrt(rho/p),
    q4 = sqrt(rho p), all positive here)."""
    rng = np.random.default_rng(50 + sd)
    for _ in range(50):
        x = np.concatenate([rng.uniform(0.5, 2.0, 1), rng.uniform(-1, 1, 3), rng.uniform(0.5, 3.0, 2),
                            rng.uniform(0.5, 2.0, 1), rng.uniform(-1, 1, 3), rng.uniform(0.5, 3.0, 2)])
        ms = rng.standard_normal(3)

        def f(x):
            G = np.empty(5)
            pt.fgpt_split_pair_gen(sd, _p(np.ascontiguousarray(x)), _p(ms), _p(G))
            return G

        def fadj(x, yb):
            xb = np.empty(12)
            pt.fgpt_split_pair_gen_adj(sd, _p(np.ascontiguousarray(x)), _p(ms), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 5, rng, hs=(2e-6, 4e-6) if sd in (5, 6) else (1e-5, 2e-5), cancel=1e-3)
        assert err is not None and err < TOL, err


@pytest.mark.parametrize("sd", [0, 4, 1, 2, 3, 5, 6])
def test_split_node_inputs_adjoint(pt, sd):
    rng = np.random.default_rng(60 + sd)
    for _ in range(30):
        s_ = _state(rng)
        x = np.array([s_[0], s_[2], s_[4], s_[5], s_[6], s_[3], s_[1]])  # rho, E, u, v, w, p, 1/rho as independent fields

        def f(x):
            q = np.empty(6)
            pt.fgpt_split_node_inputs(sd, _p(np.ascontiguousarray(x)), _p(q))
            return q

        def fadj(x, yb):
            xb = np.empty(7)
            pt.fgpt_split_node_inputs_adj(sd, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(yb)), _p(xb))
            return xb

        err = _check(f, fadj, x, 6, rng)
        assert err is not None and err < TOL, err


@pytest.mark.parametrize("sd", [1, 2, 3, 5, 6])
def test_split_surface_flux_more_adjoint(pt, sd):
    rng = np.random.default_rng(70 + sd)
    for _ in range(50):
        x = np.concatenate([_state(rng, vmax=1.6), _state(rng, vmax=1.6)])

        def f(x):
            F = np.empty(5)
            pt.fgpt_split_surface_more(sd, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])), _p(F))
            return F

        def fadj(x, yb):
            Lb, Rb = np.empty(7), np.empty(7)
            pt.fgpt_split_surface_more_adj(sd, _p(np.ascontiguousarray(x[:7])), _p(np.ascontiguousarray(x[7:])),
                                           _p(np.ascontiguousarray(yb)), _p(Lb), _p(Rb))
            return np.concatenate([Lb, Rb])

        err = _check(f, fadj, x, 5, rng, hs=(2e-6, 4e-6) if sd in (5, 6) else (1e-5, 2e-5), cancel=1e-3)
        assert err is not None and err < TOL, err


def test_entropy_variable_transforms_adjoint(pt):
    """ConsToEntropy and EntropyToCons of the Gauss split-form prolongation, transposed; EntropyToCons
    inverts ConsToEntropy."""
    rng = np.random.default_rng(40)
    for _ in range(50):
        s = _state(rng)
        U = np.array([s[0], s[0] * s[4], s[0] * s[5], s[0] * s[6], s[2]])
        W = np.empty(5)
        pt.fgpt_cons_to_entropy(KAPPA, _p(U), _p(W))
        back = np.empty(5)
        pt.fgpt_entropy_to_cons(KAPPA, _p(W), _p(back))
        assert np.allclose(back, U, rtol=1e-13, atol=1e-13)
        for fwd, adj, x in (("fgpt_cons_to_entropy", "fgpt_cons_to_entropy_adj", U), ("fgpt_entropy_to_cons", "fgpt_entropy_to_cons_adj", W)):
            def f(x, fwd=fwd):
                out = np.empty(5)
                getattr(pt, fwd)(KAPPA, _p(np.ascontiguousarray(x)), _p(out))
                return out

            def fadj(x, yb, adj=adj):
                xb = np.empty(5)
                getattr(pt, adj)(KAPPA, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(yb)), _p(xb))
                return xb

            err = _check(f, fadj, x, 5, rng)
            assert err is not None and err < TOL, (fwd, err)
