"""The Riemann solvers and two-point split fluxes of the GPU kernels (fg_common.cuh, compiled as host code in
libfgpoint.so) against the oracle's restatements of riemann.f90 and splitflux.f90, point by point on the CPU:
every solver with the weak form and with every SplitDG (SD, MO, DU, KG, PI, CH, IR), the volume fluxes of every SplitDG
in the kernels' contravariant form, and the consistency of each flux (equal states give the physical flux: the split
volume fluxes twice it, IR once, as the reference has it). Random physical states, relative bar 1e-13."""
import ctypes

import numpy as np
import pytest

from flexi_gb300 import build as fbuild
from flexi_gb300 import mesh as fmesh
from oracle import oracle as orc

KAPPA = 1.4
SPLITS = {"weak": -1, "sd": 0, "mo": 1, "du": 2, "kg": 3, "pi": 4, "ch": 5, "ir": 6}
SOLVERS = {"lf": 1, "hllc": 2, "roe": 3, "roeentropyfix": 33, "roel2": 32, "roeentropygshockfix": 34, "hll": 4, "hlle": 5, "hllem": 6,
           "ch": 7, "ir": 8, "avg": 0}
SPLIT_ONLY = {"ch", "ir", "avg"}
TOL = 1e-13


@pytest.fixture(scope="module")
def pt():
    L = ctypes.CDLL(fbuild.build_point_harness())
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.fgpt_riemann_more.argtypes = [I, I, D, D, D, P, P, P]
    L.fgpt_split_volume.argtypes = [I, D, P, P, P, P, P, P, P]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


_ORACLES = {}


def oracle_for(split, phi=5.0):
    key = (split, phi)
    if key not in _ORACLES:
        cfg = dict(N=1, nodeType=2, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=split, etaBR2=2.0,
                   etaBR2_wall=-1.0, kappa=KAPPA, R=287.058, Pr=0.72, mu0=0.0, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0,
                   riemannPhi=phi)
        _ORACLES[key] = orc.Oracle(cfg, fmesh.tgv_box(1))
    return _ORACLES[key]


def random_state(rng, mach):
    rho = rng.uniform(0.5, 2.0)
    p = rng.uniform(0.5, 2.0)
    c = np.sqrt(KAPPA * p / rho)
    v = rng.uniform(-1, 1, 3) * mach * c
    E = p / (KAPPA - 1.0) + 0.5 * rho * (v @ v)
    return rho, v, p, E


def ext(rho, v, p, E):
    """extended rotated state of riemann.f90 (0..4 cons, 5 srho, 6..8 vel, 9 p, 10 T)"""
    return np.array([rho, rho * v[0], rho * v[1], rho * v[2], E, 1.0 / rho, v[0], v[1], v[2], p, p / (rho * 287.058)])


def rot(rho, v, p, E):
    """the kernels' rotated state (rho, srho, E, p, v1, v2, v3)"""
    return np.array([rho, 1.0 / rho, E, p, v[0], v[1], v[2]])


def euler_1d(rho, v, p, E):
    return np.array([rho * v[0], rho * v[0] * v[0] + p, rho * v[0] * v[1], rho * v[0] * v[2], (E + p) * v[0]])


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("split", list(SPLITS))
@pytest.mark.parametrize("solver", list(SOLVERS))
def test_riemann_matches_oracle(pt, solver, split):
    if solver in SPLIT_ONLY and split == "weak":
        pytest.skip("split-form solver")
    sd, sid = SPLITS[split], SOLVERS[solver]
    o = oracle_for(sd, 3.0)
    rng = np.random.default_rng(100 * sid + sd + 7)
    worst = 0.0
    for k in range(60):
        mach = [0.05, 0.5, 1.5][k % 3]  # subsonic and supersonic interfaces (HLL branches, entropy fixes)
        a, b = random_state(rng, mach), random_state(rng, mach)
        Fo = o.point_riemann(sid, ext(*a), ext(*b))
        Fg = np.empty(5)
        pt.fgpt_riemann_more(sid, sd, KAPPA, 287.058, 3.0, _p(rot(*a)), _p(rot(*b)), _p(Fg))
        worst = max(worst, rel(Fg, Fo))
    assert worst <= TOL, worst


@pytest.mark.parametrize("split", [s for s in SPLITS if s != "weak"])
def test_split_volume_flux_matches_oracle(pt, split):
    sd = SPLITS[split]
    o = oracle_for(sd)
    rng = np.random.default_rng(sd + 31)
    worst = 0.0
    for _ in range(100):
        a, b = random_state(rng, 0.5), random_state(rng, 0.5)
        mR, m = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
        uR = np.array([a[0], *(a[0] * a[1]), a[3]]); pR = np.array([a[0], *a[1], a[2], 0.0])
        u = np.array([b[0], *(b[0] * b[1]), b[3]]); p = np.array([b[0], *b[1], b[2], 0.0])
        Fo = o.point_split_volume(uR, pR, u, p, mR, m)
        Fg = np.empty(5)
        pt.fgpt_split_volume(sd, KAPPA, _p(uR), _p(pR), _p(u), _p(p), _p(mR), _p(m), _p(Fg))
        worst = max(worst, rel(Fg, Fo))
    assert worst <= TOL, worst


@pytest.mark.parametrize("split", [s for s in SPLITS if s != "weak"])
def test_split_volume_flux_consistency(split):
    """Equal states: 2 m . F(u) (the factor 2 of the split form), IR: m . F(u) (splitflux.f90's IR has no factor 2).
    Symmetric in the two states."""
    sd = SPLITS[split]
    o = oracle_for(sd)
    rng = np.random.default_rng(sd + 57)
    for _ in range(20):
        rho, v, p, E = random_state(rng, 0.7)
        u = np.array([rho, *(rho * v), E]); pr = np.array([rho, *v, p, 0.0])
        m1, m2 = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
        F = o.point_split_volume(u, pr, u, pr, m1, m2)
        mm = 0.5 * (m1 + m2)
        f = np.array([rho * (v @ mm), *(rho * v * (v @ mm) + p * mm), (E + p) * (v @ mm)])
        assert rel(F, (1.0 if split == "ir" else 2.0) * f) <= 1e-13
        b = random_state(rng, 0.7)
        ub = np.array([b[0], *(b[0] * b[1]), b[3]]); pb = np.array([b[0], *b[1], b[2], 0.0])
        assert rel(o.point_split_volume(u, pr, ub, pb, m1, m2), o.point_split_volume(ub, pb, u, pr, m2, m1)) <= 1e-13


@pytest.mark.parametrize("split", list(SPLITS))
@pytest.mark.parametrize("solver", list(SOLVERS))
def test_riemann_consistency(solver, split):
    """Equal states on both sides give the physical flux F(u) (riemann.f90 solvers are consistent)."""
    if solver in SPLIT_ONLY and split == "weak":
        pytest.skip("split-form solver")
    o = oracle_for(SPLITS[split], 3.0)
    rng = np.random.default_rng(SOLVERS[solver] + 3 * SPLITS[split] + 90)
    for _ in range(20):
        s = random_state(rng, 0.8)
        F = o.point_riemann(SOLVERS[solver], ext(*s), ext(*s))
        assert rel(F, euler_1d(*s)) <= 1e-13, (F, euler_1d(*s))


def test_log_mean_series_branch():
    """GetLogMean: the series branch (|f| < 0.1) against (a - b) / (ln a - ln b); its truncation error is below 1e-8."""
    o = oracle_for(5)
    rng = np.random.default_rng(4)
    for _ in range(50):
        a = rng.uniform(0.5, 2.0)
        b = a * rng.uniform(0.83, 1.2)
        # the CH volume flux's density term equals rho_log * {u}.m: recover rho_log from it with u = 1, m = e1
        uR = np.array([a, a, 0.0, 0.0, 2.5 + 0.5 * a]); pR = np.array([a, 1.0, 0.0, 0.0, 1.0, 0.0])
        u = np.array([b, b, 0.0, 0.0, 2.5 + 0.5 * b]); p = np.array([b, 1.0, 0.0, 0.0, 1.0, 0.0])
        F = o.point_split_volume(uR, pR, u, p, np.array([1.0, 0, 0]), np.array([1.0, 0, 0]))
        exact = (a - b) / (np.log(a) - np.log(b)) if a != b else a
        assert abs(F[0] / 2.0 - exact) <= 1e-8 * exact
