"""The low-storage Runge-Kutta schemes of TimeStepByLSERKW2 (timestep.f90:82-152, tables timedisc_vars.f90:137-457).

The library's tables (fg_lserk_table) equal the oracle's restatement, the ini names map to the codes, and
the coefficients are pinned by the schemes' orders: the stability polynomial of the 2-register recursion
matches exp(z) up to z^p, and on nonautonomous nonlinear problems (stage times t + RKc dt) the global error
falls with order p. p = 3 for standardrk3-3 and toulorgerk3-7c, 4 for the others.
"""
import ctypes
import math

import numpy as np
import pytest

from flexi_gb300 import _lib
from flexi_gb300.solver import FlexiError, config_dict, config_from_ini
from oracle import oracle as orc

NAMES = ["carpenterrk4-5", "standardrk3-3", "niegemannrk4-14", "toulorgerk4-8c", "toulorgerk3-7c", "toulorgerk4-8f"]
ORDER = [4, 3, 4, 4, 3, 4]


def _table(code):
    L = _lib.load()
    st = ctypes.c_int(0)
    A, b, c, alpha, rel = np.zeros(21), np.zeros(21), np.zeros(21), np.zeros(30), ctypes.c_double(0.0)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert L.fg_lserk_table(code, ctypes.byref(st), p(A), p(b), p(c), p(alpha), ctypes.byref(rel)) == 0
    return st.value, A, b, c, alpha, rel.value


@pytest.mark.parametrize("code", range(6))
def test_tables_match_oracle_and_names(code):
    s, A, b, c, alpha, rel = _table(code)
    so, Ao, bo, co = orc.lserk_table(code)
    assert s == so and np.array_equal(A, Ao) and np.array_equal(b, bo) and np.array_equal(c, co)
    assert (alpha > 0).all() and (alpha[15:] > alpha[:15]).all() and rel >= 1.0  # GL allows the larger step
    assert config_dict(config_from_ini(f"TimeDiscMethod = {NAMES[code]}\n"))["TimeDiscMethod"] == code
    assert config_dict(config_from_ini(f"TimeDiscMethod = {NAMES[code].upper()}\n"))["TimeDiscMethod"] == code


def test_unknown_scheme_is_refused():
    L = _lib.load()
    st = ctypes.c_int(0)
    assert L.fg_lserk_table(6, ctypes.byref(st), None, None, None, None, None) != 0
    # 3-register and implicit schemes of the reference are not TimeStepByLSERKW2 schemes
    from flexi_gb300.solver import Flexi
    for name in ("ketchesonrk4-20", "esdirk3-4"):
        with pytest.raises(FlexiError):
            Flexi(config_from_ini(f"TimeDiscMethod = {name}\n"))


def _step(A, b, c, s, f, t, y, dt):
    g = np.zeros_like(y)
    for k in range(1, s + 1):
        fk = f(t + c[k] * dt, y)
        g = fk if k == 1 else fk - A[k] * g
        y = y + b[k] * dt * g
    return y


@pytest.mark.parametrize("code", range(6))
def test_stability_polynomial(code):
    s, A, b, c, _, _ = _table(code)
    # y' = z y with dt = 1, polynomials in z as coefficient arrays
    y = np.zeros(s + 1)
    y[0] = 1.0
    g = np.zeros(s + 1)
    for k in range(1, s + 1):
        zy = np.concatenate([[0.0], y[:-1]])
        g = zy if k == 1 else zy - A[k] * g
        y = y + b[k] * g
    p = ORDER[code]
    want = np.array([1.0 / math.factorial(k) for k in range(p + 1)])
    assert np.allclose(y[:p + 1], want, rtol=0, atol=1e-12), (y[:p + 1], want)


@pytest.mark.parametrize("code", range(6))
def test_order_on_nonautonomous_problems(code):
    s, A, b, c, _, _ = _table(code)
    # y1' = -2 t y1^2 (y1 = 1/(1+t^2)), y2' = y2 cos t (y2 = exp(sin t))
    f = lambda t, y: np.array([-2.0 * t * y[0] ** 2, y[1] * math.cos(t)])
    exact = np.array([1.0 / 2.0, math.exp(math.sin(1.0))])
    errs = []
    for nsteps in (10, 20, 40):
        y, t, dt = np.array([1.0, 1.0]), 0.0, 1.0 / nsteps
        for _ in range(nsteps):
            y = _step(A, b, c, s, f, t, y, dt)
            t += dt
        errs.append(np.abs(y - exact).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert (rates > ORDER[code] - 0.3).all(), (errs, rates)
