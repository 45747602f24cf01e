"""Host-side mirror of FLEXI's module interface for the DGSEM right-hand side and the LSERK stepper.

The methods keep the reference's names and meaning:
    DGTimeDerivative_weakForm(t)   src/dg/dg.f90:221
    TimeStepByLSERKW2(t, dt)       src/timedisc/timestep.f90:82 (CarpenterRK4-5, timedisc_vars.f90:199)
    CalcTimeStep()                 src/equations/navierstokes/calctimestep.f90:89
    TimeDisc(nSteps)               loop body of src/timedisc/timedisc.f90:190-212 (UpdateTimeStep, CalcForcing, TimeStep)
Arrays use FLEXI's Fortran layouts, held in numpy with reversed axes: U(1:5,0:N,0:N,0:N,1:nElems) is
an array of shape (nElems, N+1, N+1, N+1, 5). All work runs in libflexigpu.so on the GPU; a missing
library or GPU raises instead of falling back to anything else.
"""
import ctypes

import numpy as np

from . import _lib
from .mesh import BoxMesh

NODE_TYPES = {"gauss": 1, "gauss-lobatto": 2}
RIEMANN = {"avg": 0, "lf": 1, "hllc": 2, "roe": 3, "hll": 4, "hlle": 5, "hllem": 6, "ch": 7, "ir": 8, "roel2": 32, "roeentropyfix": 33,
           "roeentropygshockfix": 34, "same": -1}
SPLIT = {"none": -1, "weak": -1, "sd": 0, "mo": 1, "du": 2, "kg": 3, "pi": 4, "ch": 5, "ir": 6}


class FlexiError(RuntimeError):
    """A failed call of the C ABI; `code` is its FG_ERR_* status (0 where no call failed)."""

    def __init__(self, msg, code=0):
        super().__init__(msg)
        self.code = code


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_config(**kw) -> _lib.FgConfig:
    """fg_config with the reference defaults, overridden by keyword arguments (ini key names;
    string values accepted for NodeType, Riemann, RiemannBC, SplitDG, Lifting)."""
    L = _lib.load()
    c = _lib.FgConfig()
    L.fg_config_default(ctypes.byref(c))
    for k, v in kw.items():
        if k == "NodeType" and isinstance(v, str):
            v = NODE_TYPES[v.lower()]
        elif k in ("Riemann", "RiemannBC") and isinstance(v, str):
            v = RIEMANN[v.lower()]
        elif k == "SplitDG" and isinstance(v, str):
            v = SPLIT[v.lower()]
        elif k == "Lifting" and isinstance(v, str):
            v = {"br1": 1, "br2": 2}[v.lower()]
        elif k == "OverintegrationType" and isinstance(v, str):
            v = {"none": 0, "cutoff": 1, "conscutoff": 2}[v.lower()]
        if not hasattr(c, k):
            raise KeyError(k)
        t = type(getattr(c, k))
        setattr(c, k, t(*v) if issubclass(t, ctypes.Array) else t(v))
    return c


def config_from_ini(text: str) -> _lib.FgConfig:
    L = _lib.load()
    c = _lib.FgConfig()
    L.fg_config_default(ctypes.byref(c))
    if L.fg_config_from_ini(text.encode(), ctypes.byref(c)) != 0:
        raise FlexiError("invalid parameter file")
    return c


def config_dict(c: _lib.FgConfig) -> dict:
    d = {name: getattr(c, name) for name, _ in _lib.FgConfig._fields_}
    return {k: (tuple(v) if isinstance(v, ctypes.Array) else v) for k, v in d.items()}


class Flexi:
    """One GPU solver: configuration + mesh + state (an ensemble when the mesh has several instances)."""

    def __init__(self, cfg: _lib.FgConfig, mesh: BoxMesh = None):
        self.L = _lib.load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.L.fg_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise FlexiError(f"fg_create failed ({rc}): {self.L.fg_last_error(None).decode()}")
        self.h = h
        self.N = cfg.N
        self.n = cfg.N + 1
        if mesh is not None:
            self.build_mesh(mesh)

    def _check(self, rc, what):
        if rc != 0:
            raise FlexiError(f"{what} failed ({rc}): {self.L.fg_last_error(self.h).decode()}", rc)

    def close(self):
        if getattr(self, "h", None):
            self.L.fg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- mesh
    def build_mesh(self, m: BoxMesh, host_only_ok=False):
        """fg_build_mesh (fg_build_mesh_mortar when the mesh has mortar interfaces). host_only_ok: accept a
        failed device upload (no GPU) once the host-side preparation succeeded, so that the set-up can be
        inspected on a machine without a GPU."""
        nc = np.ascontiguousarray(m.node_coords, np.float64)
        nb = np.ascontiguousarray(m.elem_nb, np.int32)
        bt = np.ascontiguousarray(m.boundary_type, np.int32).reshape(-1)
        rs = np.ascontiguousarray(m.ref_state_prim, np.float64).reshape(-1)
        inst = None if m.elem_inst is None else np.ascontiguousarray(m.elem_inst, np.int32)
        mo = getattr(m, "mortars", None)
        mo = None if mo is None or len(mo) == 0 else np.ascontiguousarray(mo, np.int32).reshape(-1, 15)
        self._mesh_keep = (nc, nb, bt, rs, inst, mo)
        rc = self.L.fg_build_mesh_mortar(self.h, m.n_elems, m.ngeo, _p(nc), _p(nb), len(bt) // 2, _p(bt) if len(bt) else None,
                                         len(rs) // 6, _p(rs) if len(rs) else None, _p(inst) if inst is not None else None,
                                         0 if mo is None else len(mo), _p(mo) if mo is not None else None)
        if not (host_only_ok and rc == 3):  # FG_ERR_CUDA after a complete host-side set-up
            self._check(rc, "fg_build_mesh")
        self._sizes()

    def set_mesh(self, side_to_elem, elem_to_side, bc, boundary_type, ref_state_prim, Mf, Mg, Mh, sJ, NormVec, TangVec1, TangVec2, SurfElem,
                 mortar_type=None, mortar_info=None, host_only_ok=False):
        """Drop-in path: FLEXI's own processed mesh arrays (MOD_Mesh_Vars); with mortar interfaces also
        MortarType (nSides, 2) and MortarInfo (nMortars, 4, 2) (fg_set_mesh_mortar)."""
        a = [np.ascontiguousarray(x) for x in (Mf, Mg, Mh, sJ, NormVec, TangVec1, TangVec2, SurfElem)]
        s2e = np.ascontiguousarray(side_to_elem, np.int32)
        e2s = np.ascontiguousarray(elem_to_side, np.int32)
        bcv = np.ascontiguousarray(bc, np.int32)
        bt = np.ascontiguousarray(boundary_type, np.int32).reshape(-1)
        rs = np.ascontiguousarray(ref_state_prim, np.float64).reshape(-1)
        n_elems = a[3].shape[0]
        n_sides = s2e.shape[0]
        mt = None if mortar_type is None else np.ascontiguousarray(mortar_type, np.int32)
        mi = None if mortar_info is None else np.ascontiguousarray(mortar_info, np.int32).reshape(-1, 4, 2)
        n_mortars = 0 if mi is None else len(mi)
        self._mesh_keep = (a, s2e, e2s, bcv, bt, rs, mt, mi)
        rc = self.L.fg_set_mesh_mortar(self.h, n_elems, n_sides, len(bcv), _p(s2e), _p(e2s), _p(bcv) if len(bcv) else None,
                                       len(bt) // 2, _p(bt) if len(bt) else None, len(rs) // 6, _p(rs) if len(rs) else None,
                                       *[_p(x) for x in a], n_mortars, _p(mt) if n_mortars else None, _p(mi) if n_mortars else None)
        if not (host_only_ok and rc == 3):  # FG_ERR_CUDA after a complete host-side set-up
            self._check(rc, "fg_set_mesh")
        self._sizes()

    def set_face_metrics(self, Ja_Face, Ja_slave):
        """Drop-in path, split form on Gauss nodes: FLEXI's Ja_Face / Ja_slave (nSides, 0:N, 0:N, 3, 3) in C
        order of the Fortran (3,3,0:N,0:N,nSides) arrays."""
        a = np.ascontiguousarray(Ja_Face, np.float64)
        b = np.ascontiguousarray(Ja_slave, np.float64)
        self._check(self.L.fg_set_face_metrics(self.h, _p(a), _p(b)), "fg_set_face_metrics")

    def set_time(self, t):
        """fg_set_time: the device-side time of every instance (start of fg_run / fg_adjoint_forward)."""
        tt = np.ascontiguousarray(np.broadcast_to(np.asarray(t, np.float64), (max(1, getattr(self, "n_inst", 1)),)))
        self._check(self.L.fg_set_time(self.h, _p(tt)), "fg_set_time")

    def get_config(self):
        """fg_get_config: the configuration the handle runs with (BR2 turns doWeakLifting off, lifting.f90:137-139)."""
        c = _lib.FgConfig()
        self._check(self.L.fg_get_config(self.h, ctypes.byref(c)), "fg_get_config")
        return c

    def overintegrate_state(self):
        """timedisc.f90:115-123: the overintegration of U before the first time step (no-op without it)."""
        self._check(self.L.fg_overintegrate_state(self.h), "fg_overintegrate_state")

    def write_state(self, path, project="", mesh_file="", t=0.0):
        """WriteState (hdf5_output.f90:60-188): DG_Solution and the header attributes of a FLEXI state file."""
        rc = self.L.fg_write_state(self.h, str(path).encode(), project.encode(), mesh_file.encode(), float(t))
        if rc != 0:
            raise FlexiError(f"fg_write_state: {self.L.fg_io_last_error().decode()}")

    def read_state(self, path):
        """DG_Solution of a FLEXI state file with this solver's N, node type and element count; returns its Time."""
        t = ctypes.c_double(0.0)
        rc = self.L.fg_read_state(self.h, str(path).encode(), ctypes.byref(t))
        if rc != 0:
            raise FlexiError(f"fg_read_state: {self.L.fg_io_last_error().decode()}")
        return t.value

    def _sizes(self):
        s = np.zeros(5, np.int32)
        self._check(self.L.fg_get_sizes(self.h, _p(s)), "fg_get_sizes")
        self.n_elems, self.n_sides, self.n_bc_sides, _, self.n_inst = (int(v) for v in s)

    def set_instance_mu0(self, mu0):
        mu0 = np.ascontiguousarray(mu0, np.float64)
        self._check(self.L.fg_set_instance_mu0(self.h, len(mu0), _p(mu0)), "fg_set_instance_mu0")

    @property
    def ushape(self):
        return (self.n_elems, self.n, self.n, self.n, 5)

    def elem_xgp(self):
        x = np.empty((self.n_elems, self.n, self.n, self.n, 3))
        self._check(self.L.fg_get_elem_xgp(self.h, _p(x)), "fg_get_elem_xgp")
        return x

    def mesh_array(self, name):
        w = {"Mf": 0, "Mg": 1, "Mh": 2, "sJ": 3, "NormVec": 4, "TangVec1": 5, "TangVec2": 6, "SurfElem": 7}[name]
        n = self.n
        shape = {0: (self.n_elems, n, n, n, 3), 1: (self.n_elems, n, n, n, 3), 2: (self.n_elems, n, n, n, 3), 3: (self.n_elems, n, n, n),
                 4: (self.n_sides, n, n, 3), 5: (self.n_sides, n, n, 3), 6: (self.n_sides, n, n, 3), 7: (self.n_sides, n, n)}[w]
        out = np.empty(shape)
        self._check(self.L.fg_get_mesh_array(self.h, w, _p(out)), "fg_get_mesh_array")
        return out

    def side_to_elem(self):
        out = np.empty((self.n_sides, 5), np.int32)
        self._check(self.L.fg_get_side_to_elem(self.h, _p(out)), "fg_get_side_to_elem")
        return out

    # ---------------------------------------------------------------- state
    @property
    def U(self):
        out = np.empty(self.ushape)
        self._check(self.L.fg_get_state(self.h, _p(out)), "fg_get_state")
        return out

    @U.setter
    def U(self, value):
        v = np.ascontiguousarray(value, np.float64).reshape(self.ushape)
        self._check(self.L.fg_set_state(self.h, _p(v)), "fg_set_state")

    def set_state_ptr(self, host_ptr):
        """U from a raw host pointer (e.g. pinned memory); Fortran layout."""
        self._check(self.L.fg_set_state(self.h, ctypes.c_void_p(host_ptr)), "fg_set_state")

    def get_state_ptr(self, host_ptr):
        self._check(self.L.fg_get_state(self.h, ctypes.c_void_p(host_ptr)), "fg_get_state")

    # ---------------------------------------------------------------- operator and stepper
    def DGTimeDerivative_weakForm(self, t=0.0, out=None):
        Ut = np.empty(self.ushape) if out is None else out
        self._check(self.L.fg_time_derivative(self.h, float(t), _p(Ut)), "fg_time_derivative")
        return Ut

    def CalcTimeStep(self):
        dt = np.zeros(max(1, getattr(self, "n_inst", 1)))
        err = ctypes.c_int(0)
        self._check(self.L.fg_calc_timestep(self.h, _p(dt), ctypes.byref(err)), "fg_calc_timestep")
        return (float(dt[0]) if len(dt) == 1 else dt), err.value

    def dt_elem(self):
        """Per-element convective and viscous time-step limits of the last CalcTimeStep."""
        a, b = np.empty(self.n_elems), np.empty(self.n_elems)
        self._check(self.L.fg_get_dt_elem(self.h, _p(a), _p(b)), "fg_get_dt_elem")
        return a, b

    def TimeStepByLSERKW2(self, t, dt):
        tt = ctypes.c_double(t)
        self._check(self.L.fg_timestep_lserkw2(self.h, ctypes.byref(tt), float(dt)), "fg_timestep_lserkw2")
        return tt.value

    def TimeDisc(self, n_steps):
        """n_steps of the TimeDisc loop (dt from CALCTIMESTEP each step, per instance); returns times."""
        t = np.zeros(self.n_inst)
        self._check(self.L.fg_run(self.h, int(n_steps), _p(t)), "fg_run")
        return t

    def TimeDisc_to_host_ptr(self, n_steps, host_ptr):
        """TimeDisc(n_steps), then U(t_end) into the host memory at host_ptr (Fortran layout), the copy overlapped with
        the last stage (fg_run_to_host); returns the times."""
        t = np.zeros(self.n_inst)
        self._check(self.L.fg_run_to_host(self.h, int(n_steps), _p(t), ctypes.c_void_p(host_ptr)), "fg_run_to_host")
        return t

    def timedisc_state(self):
        """Per-instance state of the time loop (fg_get_timedisc_state): list of dicts with t, dt, dtMin, iter,
        atAnalyze, finished, nDtLimited."""
        n = max(1, getattr(self, "n_inst", 1))
        arr = (_lib.FgTimeDiscState * n)()
        self._check(self.L.fg_get_timedisc_state(self.h, n, arr), "fg_get_timedisc_state")
        return [{k: getattr(a, k) for k, _ in _lib.FgTimeDiscState._fields_} for a in arr]

    def gradients(self):
        n = self.n
        g = [np.empty((self.n_elems, n, n, n, 4)) for _ in range(3)]
        self._check(self.L.fg_get_gradients(self.h, _p(g[0]), _p(g[1]), _p(g[2])), "fg_get_gradients")
        return g

    # ---------------------------------------------------------------- differentiation
    def set_elem_mu_scale(self, scale):
        """Per-element viscosity multiplier (None: all ones)."""
        if scale is None:
            self._check(self.L.fg_set_elem_mu_scale(self.h, None), "fg_set_elem_mu_scale")
            return
        s = np.ascontiguousarray(scale, np.float64).reshape(self.n_elems)
        self._check(self.L.fg_set_elem_mu_scale(self.h, _p(s)), "fg_set_elem_mu_scale")

    def vjp_time_derivative(self, W, t=0.0):
        """(V, mu_bar): V = (dUt/dU)^T W at the current state, mu_bar = d<W, Ut>/d(viscosity multipliers)."""
        W = np.ascontiguousarray(W, np.float64).reshape(self.ushape)
        V = np.empty(self.ushape)
        mub = np.empty(self.n_elems)
        self._check(self.L.fg_vjp_time_derivative(self.h, float(t), _p(W), _p(V), _p(mub)), "fg_vjp_time_derivative")
        return V, mub

    def jvp_time_derivative(self, V, t=0.0, fd_order=1, eps_method=2, scaleps=1.0):
        """J V at the current state by the reference's matrix-free finite difference (implicit.f90:MatrixVector);
        the defaults are the reference's (FD_Order 1, Eps_Method 2, scaleps 1)."""
        V = np.ascontiguousarray(V, np.float64).reshape(self.ushape)
        JV = np.empty(self.ushape)
        self._check(self.L.fg_jvp_time_derivative(self.h, float(t), _p(V), _p(JV), int(fd_order), int(eps_method), float(scaleps)),
                    "fg_jvp_time_derivative")
        return JV

    def adjoint_forward(self, n_steps, dt, ckpt_every=None, snapshots=None):
        """Advances n_steps LSERK steps of fixed dt, keeping a checkpoint every ckpt_every steps, or, with
        snapshots=s, the snapshots of a binomial (revolve) schedule with s snapshot states."""
        if (ckpt_every is None) == (snapshots is None):
            raise ValueError("give either ckpt_every or snapshots")
        code = int(ckpt_every) if snapshots is None else -int(snapshots)
        self._check(self.L.fg_adjoint_forward(self.h, int(n_steps), float(dt), code), "fg_adjoint_forward")

    def adjoint_recomputed_steps(self):
        """Forward steps the last adjoint_reverse re-ran."""
        return int(self.L.fg_adjoint_recomputed_steps(self.h))

    def adjoint_reverse(self, UbarT, force_bar=False):
        """(Ubar0, mu_bar[, force_bar]) for the cotangent UbarT of the final state of the last adjoint_forward."""
        UbarT = np.ascontiguousarray(UbarT, np.float64).reshape(self.ushape)
        Ub0 = np.empty(self.ushape)
        mub = np.empty(self.n_elems)
        fb = np.empty(self.ushape[:-1]) if force_bar else None
        self._check(self.L.fg_adjoint_reverse(self.h, _p(UbarT), _p(Ub0), _p(mub), _p(fb) if force_bar else None), "fg_adjoint_reverse")
        return (Ub0, mub, fb) if force_bar else (Ub0, mub)

    def set_body_force_field(self, F):
        """Additional per-node x-momentum body force, shape (nElems, n, n, n) (None: zero)."""
        if F is None:
            self._check(self.L.fg_set_body_force_field(self.h, None), "fg_set_body_force_field")
            return
        F = np.ascontiguousarray(F, np.float64).reshape(self.ushape[:-1])
        self._check(self.L.fg_set_body_force_field(self.h, _p(F)), "fg_set_body_force_field")

    def wall_shear(self, grad=False):
        """Mean wall shear J of the current state (and dJ/dU with grad=True)."""
        J = ctypes.c_double(0.0)
        g = np.empty(self.ushape) if grad else None
        self._check(self.L.fg_wall_shear(self.h, ctypes.byref(J), _p(g) if grad else None), "fg_wall_shear")
        return (J.value, g) if grad else J.value

    def autotune(self, reps=10):
        """Times the candidate launch shapes on this mesh and state and keeps the fastest; returns the
        per-launch times (ms) and the shapes in use."""
        rep = np.full(9, np.nan)
        self._check(self.L.fg_autotune(self.h, int(reps), _p(rep)), "fg_autotune")
        ch = np.zeros(4, np.int32)
        self._check(self.L.fg_autotune_choice(self.h, _p(ch)), "fg_autotune_choice")
        names = ("prep_default", "prep_alt", "lift_default", "lift_alt", "vol_default", "vol_alt", "flux_64", "flux_128", "flux_256")
        return {"ms_per_launch": {k: (None if np.isnan(v) else float(v)) for k, v in zip(names, rep)},
                "elements_per_cta": {"prep": int(ch[0]), "lift": int(ch[1]), "vol_weak": int(ch[2])}, "flux_block": int(ch[3])}

    def set_launch_shapes(self, prep, lift, vol_weak, flux_block):
        """Explicit launch shapes (elements per CTA of prep/lift/weak volume, side-kernel block size)."""
        self._check(self.L.fg_set_launch_shapes(self.h, int(prep), int(lift), int(vol_weak), int(flux_block)), "fg_set_launch_shapes")

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self.L.fg_get_stream(self.h, ctypes.byref(s)), "fg_get_stream")
        return s.value

    def launch_count(self):
        return int(self.L.fg_launch_count(self.h))

    def debug_array(self, name):
        """Copy of a device array in the device layout (inspection only)."""
        cnt = ctypes.c_longlong(0)
        self._check(self.L.fg_debug_array(self.h, name.encode(), None, ctypes.byref(cnt)), "fg_debug_array")
        dtype = np.int32 if name in ("elemInst", "elemSide", "sideElem", "bcType") else np.float64
        out = np.empty(cnt.value, dtype)
        self._check(self.L.fg_debug_array(self.h, name.encode(), _p(out), ctypes.byref(cnt)), "fg_debug_array")
        return out

    KERNEL_CLASSES = ("prep", "lift", "flux", "vol", "dt", "other")

    def profile(self, on=True):
        self._check(self.L.fg_profile_enable(self.h, int(on)), "fg_profile_enable")

    def profile_read(self):
        ms = np.zeros(6)
        cnt = np.zeros(6, np.int64)
        self._check(self.L.fg_profile_read(self.h, _p(ms), _p(cnt)), "fg_profile_read")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_CLASSES)}


def probe_fp64_tflops():
    L = _lib.load()
    v = ctypes.c_double(0.0)
    if L.fg_probe_fp64(ctypes.byref(v)) != 0:
        raise FlexiError("fg_probe_fp64 failed: " + L.fg_last_error(None).decode())
    return v.value


def probe_fp64_pipe():
    """fg_probe_fp64_pipe: DFMA, DADD, DMUL and mixed throughput of the device's FP64 pipe (T thread-instructions/s)."""
    L = _lib.load()
    r = np.zeros(4)
    if L.fg_probe_fp64_pipe(_p(r)) != 0:
        raise FlexiError("fg_probe_fp64_pipe failed: " + L.fg_last_error(None).decode())
    return {"dfma": float(r[0]), "dadd": float(r[1]), "dmul": float(r[2]), "mixed": float(r[3])}


def probe_fp64_tensor():
    """fg_probe_fp64_tensor: FP64 tensor-core MMA throughput alone and interleaved with DFMA (TFLOP/s)."""
    L = _lib.load()
    r = np.zeros(2)
    if L.fg_probe_fp64_tensor(_p(r)) != 0:
        raise FlexiError("fg_probe_fp64_tensor failed: " + L.fg_last_error(None).decode())
    return {"dmma": float(r[0]), "dmma_with_dfma": float(r[1])}


def probe_fp64_lanes():
    """fg_probe_fp64_lanes: time (ms) of the same DFMA chains with 32, 16, 8, 4 and 1 active lanes per warp."""
    L = _lib.load()
    r = np.zeros(5)
    if L.fg_probe_fp64_lanes(_p(r)) != 0:
        raise FlexiError("fg_probe_fp64_lanes failed: " + L.fg_last_error(None).decode())
    return {str(k): float(v) for k, v in zip((32, 16, 8, 4, 1), r)}

