"""ctypes front-end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle restates FLEXI v25.10's DGSEM Navier-Stokes right-hand side (src/dg/dg.f90:221-678),
its mesh/metric preprocessing (src/mesh/metrics.f90, mappings.f90) and the LSERK stepper
(src/timedisc/timestep.f90:82-152) in C++ (basis.hpp, mesh.hpp, dg.hpp, oracle_capi.cpp).
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use it, and only as the
checker / the timed CPU baseline. The product (flexi_gb300, libflexigpu.so) never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

NT_GAUSS, NT_GL, NT_CL, NT_VISU = 1, 2, 3, 4


class OrcConfig(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("nodeType", ctypes.c_int), ("riemann", ctypes.c_int), ("riemannBC", ctypes.c_int),
                ("lifting", ctypes.c_int), ("weakLifting", ctypes.c_int), ("consLifting", ctypes.c_int), ("splitDG", ctypes.c_int),
                ("etaBR2", ctypes.c_double), ("etaBR2_wall", ctypes.c_double), ("kappa", ctypes.c_double), ("R", ctypes.c_double),
                ("Pr", ctypes.c_double), ("mu0", ctypes.c_double), ("CFLScale", ctypes.c_double), ("DFLScale", ctypes.c_double),
                ("doTCSource", ctypes.c_int), ("dpdx", ctypes.c_double), ("overintType", ctypes.c_int), ("NUnder", ctypes.c_int),
                ("iniExactFunc", ctypes.c_int), ("advVel", ctypes.c_double * 3), ("iniFrequency", ctypes.c_double),
                ("iniAmplitude", ctypes.c_double), ("timeDisc", ctypes.c_int), ("riemannPhi", ctypes.c_double)]

# keys a configuration may leave out (defaults of the reference: no overintegration, NUnder = N; no source term,
# IniFrequency 1, IniAmplitude 0.1 of exact function 4)
_OPTIONAL = {"overintType": 0, "NUnder": -1, "iniExactFunc": 0, "advVel": (0.0, 0.0, 0.0), "iniFrequency": 1.0, "iniAmplitude": 0.1,
             "timeDisc": 0, "riemannPhi": 5.0}


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        _lib.orc_create.restype = P
        _lib.orc_create.argtypes = [ctypes.POINTER(OrcConfig), ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, P, ctypes.c_int, P,
                                    ctypes.c_int, P]
        _lib.orc_destroy.argtypes = [P]
        _lib.orc_last_error.restype = ctypes.c_char_p
        for f in ("orc_set_state", "orc_get_state"):
            getattr(_lib, f).argtypes = [P, P]
        _lib.orc_time_derivative.argtypes = [P, ctypes.c_double, P]
        _lib.orc_timestep.argtypes = [P, P, ctypes.c_double]
        _lib.orc_calc_timestep.argtypes = [P, P]
        _lib.orc_calc_timestep.restype = ctypes.c_double
        _lib.orc_point_riemann.argtypes = [P, ctypes.c_int, P, P, P]
        _lib.orc_point_split_volume.argtypes = [P, P, P, P, P, P, P, P]
        _lib.orc_bulk_velocity.argtypes = [P]
        _lib.orc_bulk_velocity.restype = ctypes.c_double
        _lib.orc_set_bulk_velocity.argtypes = [P, ctypes.c_double]
        _lib.orc_set_mu_scale.argtypes = [P, P]
        _lib.orc_jvp.argtypes = [P, P, P]
        _lib.orc_jvp_solve.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_double, P]
        _lib.orc_set_force_field.argtypes = [P, P]
        _lib.orc_fd_jvp.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double, P]
        _lib.orc_sizes.argtypes = [P, P]
        _lib.orc_mesh_array.argtypes = [P, ctypes.c_int, P]
        _lib.orc_mesh_array.restype = ctypes.c_longlong
        _lib.orc_mesh_iarray.argtypes = [P, ctypes.c_int, P]
        _lib.orc_mesh_iarray.restype = ctypes.c_longlong
        _lib.orc_get_gradients.argtypes = [P, ctypes.c_int, P]
        _lib.orc_flops_per_dof_stage.argtypes = [P]
        _lib.orc_flops_per_dof_stage.restype = ctypes.c_double
        _lib.orc_flops_breakdown.argtypes = [P, P]
        _lib.orc_lserk_table.argtypes = [ctypes.c_int, P, P, P, P]
        _lib.orc_set_threads.argtypes = [ctypes.c_int]
        _lib.orc_max_threads.restype = ctypes.c_int
        _lib.orc_nodes_and_weights.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P]
        _lib.orc_derivative_matrix.argtypes = [ctypes.c_int, ctypes.c_int, P]
        _lib.orc_mappings.argtypes = [ctypes.c_int, P, P]
        _lib.orc_prolong_unittest.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]
        _lib.orc_surfint_unittest.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]
        _lib.orc_surfint_split_unittest.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P]
        _lib.orc_overintegrate_state.argtypes = [P]
        _lib.orc_tgv_exact.argtypes = [ctypes.c_int, P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, P]
        _lib.orc_tgv_analysis.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double, P]
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_config(cfg: dict) -> OrcConfig:
    c = OrcConfig()
    for name, _ in OrcConfig._fields_:
        v = cfg[name] if name in cfg else _OPTIONAL[name]
        if name == "advVel":
            v = (ctypes.c_double * 3)(*v)
        setattr(c, name, v)
    return c


class Oracle:
    """CPU restatement of FLEXI's operator on one mesh. Arrays use FLEXI's Fortran layouts, stored in
    numpy as C-contiguous arrays with reversed axes, e.g. U -> shape (nElems, n, n, n, 5)."""

    def __init__(self, cfg: dict, mesh):
        L = lib()
        self.cfg = dict(cfg)
        self._c = make_config(cfg)
        nc = np.ascontiguousarray(mesh.node_coords, dtype=np.float64)
        nb = np.ascontiguousarray(mesh.elem_nb, dtype=np.int32)
        bt = np.ascontiguousarray(mesh.boundary_type, dtype=np.int32).reshape(-1)
        rs = np.ascontiguousarray(mesh.ref_state_prim, dtype=np.float64).reshape(-1)
        self._keep = (nc, nb, bt, rs)
        mo = getattr(mesh, "mortars", None)
        mo = np.zeros((0, 15), np.int32) if mo is None else np.ascontiguousarray(mo, np.int32).reshape(-1, 15)
        self.h = L.orc_create(ctypes.byref(self._c), mesh.n_elems, mesh.ngeo, _p(nc), _p(nb), len(bt) // 2, _p(bt), len(rs) // 6, _p(rs),
                              len(mo), _p(mo) if len(mo) else None)
        if not self.h:
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        s = np.zeros(4, np.int32)
        L.orc_sizes(self.h, _p(s))
        self.n_elems, self.n_sides, self.n_bc_sides, self.N = (int(x) for x in s)
        self.n = self.N + 1

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def ushape(self):
        return (self.n_elems, self.n, self.n, self.n, 5)

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.ushape)
        lib().orc_set_state(self.h, _p(U))

    def get_state(self):
        U = np.empty(self.ushape)
        lib().orc_get_state(self.h, _p(U))
        return U

    def time_derivative(self, t=0.0):
        Ut = np.empty(self.ushape)
        if lib().orc_time_derivative(self.h, t, _p(Ut)) != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return Ut

    def timestep(self, t, dt):
        tt = ctypes.c_double(t)
        if lib().orc_timestep(self.h, ctypes.byref(tt), dt) != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return tt.value

    def set_mu_scale(self, scale):
        """Per-element viscosity multiplier (None: all ones)."""
        if scale is None:
            lib().orc_set_mu_scale(self.h, None)
            return
        self._mu_scale = np.ascontiguousarray(scale, dtype=np.float64).reshape(self.n_elems)
        lib().orc_set_mu_scale(self.h, _p(self._mu_scale))

    def jvp(self, V):
        """Exact J V of the time derivative at the current state (dual-number instantiation)."""
        V = np.ascontiguousarray(V, dtype=np.float64).reshape(self.ushape)
        JV = np.empty(self.ushape)
        if lib().orc_jvp(self.h, _p(V), _p(JV)) != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return JV

    def set_force_field(self, F):
        """Additional per-node x-momentum body force, shape (nElems, n, n, n) (None: none)."""
        if F is None:
            lib().orc_set_force_field(self.h, None)
            return
        self._force = np.ascontiguousarray(F, dtype=np.float64).reshape(self.ushape[:-1])
        lib().orc_set_force_field(self.h, _p(self._force))

    def jvp_solve(self, V, n_steps, dt, d_scale=None, d_force=None):
        """Exact tangent of n_steps LSERK steps of fixed dt (dual numbers, bulk velocity included): the
        directional derivative of U(t_end) along V (initial state), d_scale (viscosity multipliers) and
        d_force (body-force field); any of them may be None."""
        Vp = None if V is None else np.ascontiguousarray(V, dtype=np.float64).reshape(self.ushape)
        Sp = None if d_scale is None else np.ascontiguousarray(d_scale, dtype=np.float64).reshape(self.n_elems)
        Fp = None if d_force is None else np.ascontiguousarray(d_force, dtype=np.float64).reshape(self.ushape[:-1])
        JV = np.empty(self.ushape)
        if lib().orc_jvp_solve(self.h, None if Vp is None else _p(Vp), None if Sp is None else _p(Sp), None if Fp is None else _p(Fp),
                               int(n_steps), float(dt), _p(JV)) != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return JV

    def fd_jvp(self, V, fd_order=2, eps_method=1, scaleps=1.0):
        """Matrix-free finite-difference J V as the reference's implicit solver forms it
        (src/implicit/implicit.f90:MatrixVector with the step size of InitImplicit)."""
        V = np.ascontiguousarray(V, dtype=np.float64).reshape(self.ushape)
        JV = np.empty(self.ushape)
        if lib().orc_fd_jvp(self.h, _p(V), fd_order, eps_method, scaleps, _p(JV)) != 0:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return JV

    def calc_timestep(self):
        err = ctypes.c_int(0)
        dt = lib().orc_calc_timestep(self.h, ctypes.byref(err))
        return dt, err.value

    def point_riemann(self, solver, L, R):
        """riemann.f90 solver `solver` on extended rotated states (11 values each) with this oracle's configuration."""
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        F = np.empty(5)
        lib().orc_point_riemann(self.h, int(solver), _p(L), _p(R), _p(F))
        return F

    def point_split_volume(self, uR, pR, u, p, mR, m):
        """splitflux.f90 two-point volume flux of this oracle's SplitDG (node states U(5), UPrim(6), metric vectors(3))."""
        a = [np.ascontiguousarray(x, np.float64) for x in (uR, pR, u, p, mR, m)]
        F = np.empty(5)
        lib().orc_point_split_volume(self.h, *[_p(x) for x in a], _p(F))
        return F

    def bulk_velocity(self):
        return lib().orc_bulk_velocity(self.h)

    def set_bulk_velocity(self, v):
        lib().orc_set_bulk_velocity(self.h, v)

    _MESH_ARRAYS = {"Mf": 0, "Mg": 1, "Mh": 2, "sJ": 3, "NormVec": 4, "TangVec1": 5, "TangVec2": 6, "SurfElem": 7,
                    "Face_xGP": 8, "Elem_xGP": 9, "wGPVol": 10, "JaN_master": 12, "JaN_slave": 13}

    def mesh_array(self, name):
        w = self._MESH_ARRAYS[name]
        cnt = lib().orc_mesh_array(self.h, w, None)
        out = np.empty(cnt)
        lib().orc_mesh_array(self.h, w, _p(out))
        n = self.n
        shapes = {"Mf": (self.n_elems, n, n, n, 3), "Mg": (self.n_elems, n, n, n, 3), "Mh": (self.n_elems, n, n, n, 3),
                  "sJ": (self.n_elems, n, n, n), "NormVec": (self.n_sides, n, n, 3), "TangVec1": (self.n_sides, n, n, 3),
                  "TangVec2": (self.n_sides, n, n, 3), "SurfElem": (self.n_sides, n, n), "Face_xGP": (self.n_sides, n, n, 3),
                  "Elem_xGP": (self.n_elems, n, n, n, 3), "wGPVol": (n, n, n), "JaN_master": (self.n_sides, n, n, 3),
                  "JaN_slave": (self.n_sides, n, n, 3)}
        return out.reshape(shapes[name])

    def volume(self):
        out = np.zeros(1)
        lib().orc_mesh_array(self.h, 11, _p(out))
        return float(out[0])

    def mesh_iarray(self, name):
        w = {"SideToElem": 0, "ElemToSide": 1, "BC": 2, "MortarType": 3, "MortarInfo": 4}[name]
        cnt = lib().orc_mesh_iarray(self.h, w, None)
        out = np.empty(max(cnt, 1), np.int32)
        lib().orc_mesh_iarray(self.h, w, _p(out))
        out = out[:cnt]
        if name == "SideToElem":
            return out.reshape(self.n_sides, 5)
        if name == "ElemToSide":
            return out.reshape(self.n_elems, 6, 2)
        if name == "MortarType":
            return out.reshape(self.n_sides, 2)
        if name == "MortarInfo":
            return out.reshape(-1, 4, 2)
        return out

    def gradients(self):
        n = self.n
        g = [np.empty((self.n_elems, n, n, n, 4)) for _ in range(3)]
        for d in range(3):
            lib().orc_get_gradients(self.h, d, _p(g[d]))
        return g

    def overintegrate_state(self):
        """timedisc.f90:115-123: the overintegration of U before the first time step."""
        lib().orc_overintegrate_state(self.h)

    def flops_per_dof_stage(self):
        return lib().orc_flops_per_dof_stage(self.h)

    def flops_breakdown(self):
        """Algorithmic flops per DOF of one LSERK stage by kernel class: prep, lift, flux, vol (incl. the
        register update), total."""
        out = np.zeros(5)
        lib().orc_flops_breakdown(self.h, _p(out))
        return dict(zip(("prep", "lift", "flux", "vol", "total"), out.tolist()))


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return lib().orc_max_threads()


def lserk_table(code):
    """(stages, A, b, c) of the oracle's low-storage scheme `code` (1-based stage arrays of length 21)."""
    st = ctypes.c_int(0)
    A, b, c = np.zeros(21), np.zeros(21), np.zeros(21)
    if lib().orc_lserk_table(int(code), ctypes.byref(st), _p(A), _p(b), _p(c)) != 0:
        raise ValueError(f"no low-storage scheme {code}")
    return st.value, A, b, c


def nodes_and_weights(N, node_type):
    x, w, wb = np.zeros(N + 1), np.zeros(N + 1), np.zeros(N + 1)
    lib().orc_nodes_and_weights(N, node_type, _p(x), _p(w), _p(wb))
    return x, w, wb


def derivative_matrix(N, node_type):
    """D(i,l) returned as a numpy array D[i, l]."""
    D = np.zeros((N + 1) * (N + 1))
    lib().orc_derivative_matrix(N, node_type, _p(D))
    return D.reshape(N + 1, N + 1).T.copy()


def mappings(N):
    n = N + 1
    S2V2 = np.zeros((6, 5, n, n, 2), np.int32)
    S2V = np.zeros((6, 5, n, n, n, 3), np.int32)
    lib().orc_mappings(N, _p(S2V2), _p(S2V))
    return S2V2, S2V


def prolong_unittest(N, node_type, side_to_elem, s2v2, Lm, Lp, Uvol):
    n = N + 1
    nS = side_to_elem.shape[0]
    s2e = np.ascontiguousarray(side_to_elem, np.int32)
    s2v2 = np.ascontiguousarray(s2v2, np.int32)
    Um = np.zeros((nS, n, n))
    lib().orc_prolong_unittest(N, node_type, nS, _p(s2e), _p(s2v2), _p(np.ascontiguousarray(Lm)), _p(np.ascontiguousarray(Lp)),
                               _p(np.ascontiguousarray(Uvol)), _p(Um))
    return Um


def surfint_unittest(N, node_type, side_to_elem, s2v2, LhM, LhP, Flux):
    n = N + 1
    nS = side_to_elem.shape[0]
    s2e = np.ascontiguousarray(side_to_elem, np.int32)
    s2v2 = np.ascontiguousarray(s2v2, np.int32)
    Ut = np.zeros((n, n, n))
    lib().orc_surfint_unittest(N, node_type, nS, _p(s2e), _p(s2v2), _p(np.ascontiguousarray(LhM)), _p(np.ascontiguousarray(LhP)),
                               _p(np.ascontiguousarray(Flux)), _p(Ut))
    return Ut


def surfint_split_unittest(N, side_to_elem, Lm, Lp, LhM, LhP, Flux):
    """Split-Gauss SurfInt of the reference's unit test (unit states and metrics, SD split flux)."""
    n = N + 1
    nS = side_to_elem.shape[0]
    s2e = np.ascontiguousarray(side_to_elem, np.int32)
    Ut = np.zeros((n, n, n))
    args = [np.ascontiguousarray(a, np.float64) for a in (Lm, Lp, LhM, LhP, Flux)]
    lib().orc_surfint_split_unittest(N, nS, _p(s2e), *[_p(a) for a in args], _p(Ut))
    return Ut


def tgv_exact(x, mach=0.1, kappa=1.4, R=71.42857, ini_const_dens=True):
    x = np.ascontiguousarray(x, np.float64)
    pts = x.reshape(-1, 3)
    U = np.empty((pts.shape[0], 5))
    lib().orc_tgv_exact(pts.shape[0], _p(pts), mach, kappa, R, int(ini_const_dens), _p(U))
    return U.reshape(x.shape[:-1] + (5,))


def tgv_analysis(N, node_type, sJ, U, grads, n_analyze, kappa, R, mu0):
    out = np.zeros(15)
    sJ = np.ascontiguousarray(sJ)
    U = np.ascontiguousarray(U)
    g = [np.ascontiguousarray(a) for a in grads]
    lib().orc_tgv_analysis(N, node_type, sJ.shape[0], _p(sJ), _p(U), _p(g[0]), _p(g[1]), _p(g[2]), n_analyze, kappa, R, mu0, _p(out))
    return out
