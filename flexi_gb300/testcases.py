"""Initial states of the benchmark cases.

* Taylor-Green vortex: src/testcase/taylorgreenvortex/testcase.f90:ExactFuncTestcase (:176-219) with
  rho0 = U0 = 1, p0 = (U0/Ma)^2/kappa*rho0 (:102-107), IniConstDens (constant density, the reference
  default, :62-64) or constant temperature T0 = p0/(rho0*R).
* Isentropic (Shu) vortex on a periodic box, as a second ensemble member type.
* Channel: laminar Poiseuille profile plus seeded random perturbation (a synthetic start for the
  wall-bounded case; the reference channel testcase starts from a turbulent mean profile).
"""
import numpy as np


def prim_to_cons(prim, kappa):
    rho, u, v, w, p = prim[..., 0], prim[..., 1], prim[..., 2], prim[..., 3], prim[..., 4]
    U = np.empty(prim.shape[:-1] + (5,))
    U[..., 0] = rho
    U[..., 1] = rho * u
    U[..., 2] = rho * v
    U[..., 3] = rho * w
    U[..., 4] = p / (kappa - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return U


def tgv_state(x, mach=0.1, kappa=1.4, R=71.42857, ini_const_dens=True):
    """x: (..., 3) solution coordinates -> conservative U (..., 5)."""
    rho0, U0 = 1.0, 1.0
    p0 = (U0 / mach) ** 2 / kappa * rho0
    T0 = p0 / (rho0 * R)
    X, Y, Z = x[..., 0], x[..., 1], x[..., 2]
    prim = np.zeros(x.shape[:-1] + (6,))
    prim[..., 1] = U0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    prim[..., 2] = -U0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    prim[..., 4] = p0 + (rho0 * U0 ** 2) / 16.0 * (np.cos(2 * X) * np.cos(2.0 * Z) + 2.0 * np.cos(2.0 * Y) + 2.0 * np.cos(2.0 * X)
                                                   + np.cos(2 * Y) * np.cos(2.0 * Z))
    if ini_const_dens:
        prim[..., 0] = rho0
        prim[..., 5] = prim[..., 4] / (prim[..., 0] * R)
    else:
        prim[..., 5] = T0
        prim[..., 0] = prim[..., 4] / (T0 * R)
    # eos.f90:PrimToCons
    U = np.empty(x.shape[:-1] + (5,))
    U[..., 0] = prim[..., 0]
    U[..., 1:4] = prim[..., 1:4] * prim[..., 0:1]
    U[..., 4] = 1.0 / (kappa - 1.0) * prim[..., 4] + 0.5 * (U[..., 1] * prim[..., 1] + U[..., 2] * prim[..., 2] + U[..., 3] * prim[..., 3])
    return U


def shu_vortex_state(x, mach=0.1, kappa=1.4, eps=5.0, center=(0.0, 0.0), period=2.0 * np.pi):
    """Isentropic vortex (Shu) in the x-y plane on a periodic box, background at rest."""
    X = (x[..., 0] - center[0] + 0.5 * period) % period - 0.5 * period
    Y = (x[..., 1] - center[1] + 0.5 * period) % period - 0.5 * period
    r2 = X * X + Y * Y
    p_inf = 1.0 / (kappa * mach * mach)
    du = eps / (2.0 * np.pi) * np.exp(0.5 * (1.0 - r2))
    dT = -(kappa - 1.0) * eps * eps / (8.0 * kappa * np.pi * np.pi) * np.exp(1.0 - r2)
    T = p_inf + dT  # rho_inf = 1 and p = rho*T, so T_inf = p_inf
    rho = (T / p_inf) ** (1.0 / (kappa - 1.0))
    p = rho * T
    prim = np.zeros(x.shape[:-1] + (6,))
    prim[..., 0] = rho
    prim[..., 1] = -Y * du
    prim[..., 2] = X * du
    prim[..., 4] = p
    return prim_to_cons(prim, kappa)


def channel_state(x, mach=0.1, kappa=1.4, R=1.0, t_wall=1.0, noise=0.05, seed=0):
    """Laminar Poiseuille profile u = 1.5 * U_b * (1 - y^2) (U_b = 1) plus seeded relative noise."""
    rng = np.random.default_rng(seed)
    y = x[..., 1]
    p0 = 1.0 / (kappa * mach * mach)
    rho0 = p0 / (R * t_wall)
    u = 1.5 * (1.0 - y * y)
    prim = np.zeros(x.shape[:-1] + (6,))
    prim[..., 0] = rho0
    prim[..., 1] = u * (1.0 + noise * rng.standard_normal(y.shape))
    prim[..., 2] = noise * u * rng.standard_normal(y.shape)
    prim[..., 3] = noise * u * rng.standard_normal(y.shape)
    prim[..., 4] = p0
    return prim_to_cons(prim, kappa)


def sine_wave_state(x, t=0.0, adv_vel=(0.3, 0.3, 0.3), frequency=1.0, amplitude=0.1):
    """exactfunc.f90 CASE(4), the oblique sine wave of the convergence tests (3D): rho = m1 = m2 = m3 =
    2 + A sin(omega (x+y+z) - a t), E = rho^2, omega = pi * frequency, a = 2 pi adv_vel[0]. With its source
    term (CalcSource CASE(4)) it solves the Navier-Stokes equations exactly."""
    x = np.asarray(x, np.float64)
    om = np.pi * frequency
    a = adv_vel[0] * 2.0 * np.pi
    g = 2.0 + amplitude * np.sin(om * x.sum(axis=-1) - a * t)
    U = np.empty(x.shape[:-1] + (5,))
    U[..., 0:4] = g[..., None]
    U[..., 4] = g * g
    return U
