"""Shared case definitions for the parity tests (configurations, meshes, initial states)."""
import numpy as np

from flexi_gb300 import mesh as fmesh
from flexi_gb300 import testcases
from flexi_gb300.solver import Flexi, make_config, config_dict
from oracle import oracle as orc

NAMES = {"lf": 1, "hllc": 2, "roe": 3, "roeentropyfix": 33}


def product_cfg(**kw):
    return make_config(**kw)


def oracle_cfg(c):
    d = config_dict(c)
    return dict(N=d["N"], nodeType=d["NodeType"], riemann=d["Riemann"], riemannBC=d["RiemannBC"], lifting=d["Lifting"],
                weakLifting=d["doWeakLifting"], consLifting=d["doConservativeLifting"], splitDG=d["SplitDG"], etaBR2=d["etaBR2"],
                etaBR2_wall=d["etaBR2_wall"], kappa=d["kappa"], R=d["R"], Pr=d["Pr"], mu0=d["mu0"], CFLScale=d["CFLScale"],
                DFLScale=d["DFLScale"], doTCSource=d["doTCSource"], dpdx=d["dpdx"], overintType=d["OverintegrationType"],
                NUnder=d["NUnder"], iniExactFunc=d["IniExactFunc"], advVel=d["AdvVel"], iniFrequency=d["IniFrequency"],
                iniAmplitude=d["IniAmplitude"], timeDisc=d["TimeDiscMethod"], riemannPhi=d["RiemannPhiFactor"])


def perturb_state(U, seed=0, amp=0.05):
    """Seeded random perturbation of a state (density and pressure stay positive) so that no component
    of the time derivative vanishes identically, as the density rate of the constant-density TGV does."""
    rng = np.random.default_rng(seed)
    U = U.copy()
    rho = U[..., 0] * (1.0 + amp * rng.uniform(-1, 1, U.shape[:-1]))
    vel = U[..., 1:4] / U[..., 0:1] + amp * rng.uniform(-1, 1, U.shape[:-1] + (3,))
    ekin_old = 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / U[..., 0]
    eint = (U[..., 4] - ekin_old) * (1.0 + amp * rng.uniform(-1, 1, U.shape[:-1]))
    U[..., 0] = rho
    U[..., 1:4] = rho[..., None] * vel
    U[..., 4] = eint + 0.5 * rho * (vel ** 2).sum(-1)
    return U


def tgv_pair(c, n_elem=4, ngeo=1, perturb=0.0, seed=0, mach=0.1, noise=0.05):
    m = fmesh.tgv_box(n_elem, ngeo=ngeo, perturb=perturb, seed=seed)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = testcases.tgv_state(f.elem_xgp(), mach=mach, kappa=c.kappa, R=c.R)
    if noise:
        U0 = perturb_state(U0, seed=seed + 11, amp=noise)
    f.U = U0
    o.set_state(U0)
    return f, o, U0


def channel_pair(c, nelems=(4, 4, 2), ngeo=2, seed=0, t_wall=1.0):
    m = fmesh.channel_box(nelems, beta=1.5, ngeo=ngeo, t_wall=t_wall, rho_wall=1.0, p_wall=1.0)
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    U0 = testcases.channel_state(f.elem_xgp(), mach=0.1, kappa=c.kappa, R=c.R, t_wall=t_wall, noise=0.05, seed=seed)
    f.U = U0
    o.set_state(U0)
    return f, o, U0


def rel_err(a, b):
    """max over variables of max|a-b| / max|b| (per conservative variable)."""
    num = np.abs(a - b).reshape(-1, 5).max(axis=0)
    den = np.abs(b).reshape(-1, 5).max(axis=0)
    return float((num / np.maximum(den, 1e-300)).max())


def _lagrange(xs, x):
    L = np.ones((len(x), len(xs)))
    for j in range(len(xs)):
        for m in range(len(xs)):
            if m != j:
                L[:, j] *= (x - xs[m]) / (xs[j] - xs[m])
    return L


def l2_error(N, node_type, x, sJ, U, U_exact_fn, n_analyze=10):
    """analyze.f90:CalcErrors on affine elements: the state interpolated from the N solution nodes to
    n_analyze+1 Gauss-Lobatto points, L2 = sqrt(sum w J |U - U_exact|^2 / volume) per variable. x, U with
    reversed axes (nElems, n, n, n, 3|5), sJ (nElems, n, n, n)."""
    xs = orc.nodes_and_weights(N, node_type)[0]
    xa, wa = orc.nodes_and_weights(n_analyze, orc.NT_GL)[:2]
    I = _lagrange(np.asarray(xs), np.asarray(xa))
    ip = lambda A: np.einsum('ai,bj,ck,eijkv->eabcv', I, I, I, A)
    J = ip((1.0 / sJ)[..., None])[..., 0]
    W = np.einsum('a,b,c->abc', wa, wa, wa) * J
    err = ip(U) - U_exact_fn(ip(x))
    return np.sqrt((err ** 2 * W[..., None]).sum(axis=(0, 1, 2, 3)) / W.sum())
