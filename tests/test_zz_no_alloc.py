"""fg_time_derivative_noalloc (allocation-free right-hand side) against fg_time_derivative and the oracle.

The allocation-free entry point exists for callers that cannot let a library allocate device memory: host codes whose
device memory all comes from their own pool or caching allocator, and time loops that must not allocate once they run.
It takes caller-owned device arrays and keeps its intermediates in a static device scratch array. Each case evaluates it
twice in a row on two different states and compares each result with the handle-based fg_time_derivative on the same
state and with the CPU oracle: max abs difference per conservative variable, normalised by that variable's max |Ut|,
within 1e-12. The allocation-free path forms the metric x 1/J products inside its kernels where the handle uses products
formed at mesh upload, so the two differ by round-off and the oracle is the common reference. This file is collected last
so that it also runs after every other GPU test in one process; it passes alone in a fresh process as well."""
import ctypes

import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, rel_err
from flexi_gb300 import _lib, mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, make_config
from oracle import oracle as orc

UT_TOL = 1e-12


def _device_mesh(f):
    """fg_device_mesh of a Flexi handle's mesh (its own device tables copied out), in caller-owned torch device memory."""
    import torch

    nb = max(f.n_bc_sides, 1)
    bct = f.debug_array("bcType") if f.n_bc_sides else np.full(1, 4, np.int32)
    bcw = f.debug_array("bcTwall") if f.n_bc_sides else np.ones(1)
    keep = {
        "elemSide": torch.from_numpy(f.debug_array("elemSide")).cuda(),
        "sideElem": torch.from_numpy(f.debug_array("sideElem")).cuda(),
        "metr": torch.from_numpy(f.debug_array("metr")).cuda(),
        "sJ": torch.from_numpy(f.debug_array("sJ")).cuda(),
        "geo": torch.from_numpy(f.debug_array("geo")).cuda(),
        "bcType": torch.from_numpy(np.ascontiguousarray(bct[:nb])).cuda(),
        "bcTwall": torch.from_numpy(np.ascontiguousarray(bcw[:nb])).cuda(),
    }
    m = _lib.FgDeviceMesh(f.n_elems, f.n_sides, f.n_bc_sides, *[keep[k].data_ptr() for k in
                                                                  ("elemSide", "sideElem", "metr", "sJ", "geo", "bcType", "bcTwall")])
    return m, keep


def _to_dev_layout(U, n_elems, n3):
    """(nElems, k, j, i, 5) -> device layout [e][5][n3]."""
    return np.ascontiguousarray(U.reshape(n_elems, n3, 5).transpose(0, 2, 1))


def _channel_mixed_walls(t_wall):
    """Channel box whose lower wall is isothermal (BC type 4) and upper wall adiabatic (BC type 3)."""
    m = fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2, t_wall=t_wall)
    m.boundary_type = np.array([[4, 1], [3, 1]], np.int32)
    upper = m.elem_nb[:, 3, 2] == 1  # local side ETA_PLUS (4) of the top elements
    m.elem_nb[upper, 3, 2] = 2
    return m


CASES = {
    # benchmark discretisation on a curved periodic box: N=7 Gauss-Lobatto, split form (Pirozzoli), BR2
    "gl7_split_pi_br2_curved": (dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2"), "tgv"),
    # weak form on Gauss nodes with isothermal no-slip walls, BR1
    "gauss3_weak_br1_channel": (dict(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1"), "channel"),
    # split form SD on Gauss-Lobatto nodes, BR2 with its wall penalty, an isothermal and an adiabatic wall
    "gl3_split_sd_br2_mixed_walls": (dict(N=3, NodeType="gauss-lobatto", SplitDG="sd", Riemann="hllc", Lifting="br2", etaBR2_wall=1.5),
                                     "mixed"),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_matches_handle_two_calls(name):
    import torch

    kw, kind = CASES[name]
    c = make_config(mu0=2e-3, **kw)
    t_wall = 1.0
    if kind == "tgv":
        m = fmesh.tgv_box(3, ngeo=2, perturb=0.05, seed=3)
    elif kind == "channel":
        m = fmesh.channel_box((4, 4, 2), beta=1.5, ngeo=2, t_wall=t_wall)
    else:
        m = _channel_mixed_walls(t_wall)
    f = Flexi(c, m)
    xgp = f.elem_xgp()
    if kind == "tgv":
        base = testcases.tgv_state(xgp, mach=0.1, kappa=c.kappa, R=c.R)
    else:
        base = testcases.channel_state(xgp, mach=0.1, kappa=c.kappa, R=c.R, t_wall=t_wall, noise=0.0, seed=0)
    states = [perturb_state(base, seed=21, amp=0.05), perturb_state(base, seed=22, amp=0.05)]
    if kind != "tgv":
        assert f.n_bc_sides > 0
    if kind == "mixed":
        assert set(f.debug_array("bcType").tolist()) == {3, 4}
    n3 = f.n ** 3
    L = _lib.load()
    dmesh, keep = _device_mesh(f)
    o = orc.Oracle(oracle_cfg(c), m)
    refs, orcs = [], []
    for U in states:
        f.U = U
        refs.append(f.DGTimeDerivative_weakForm(0.0))
        o.set_state(U)
        orcs.append(o.time_derivative(0.0))
    U_devs = [torch.from_numpy(_to_dev_layout(U, f.n_elems, n3)).cuda() for U in states]
    Ut_devs = [torch.full_like(u, float("nan")) for u in U_devs]
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free = []
    for U_dev, Ut_dev in zip(U_devs, Ut_devs):  # two calls in a row
        before = torch.cuda.mem_get_info()[0]
        rc = L.fg_time_derivative_noalloc(ctypes.byref(c), ctypes.byref(dmesh), ctypes.c_void_p(U_dev.data_ptr()),
                                          ctypes.c_void_p(Ut_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.fg_last_error(None)
        torch.cuda.synchronize()
        free.append((before, torch.cuda.mem_get_info()[0]))
    for call, (ref, ref_o, Ut_dev) in enumerate(zip(refs, orcs, Ut_devs)):
        got = Ut_dev.cpu().numpy().reshape(f.n_elems, 5, n3).transpose(0, 2, 1).reshape(ref.shape)
        assert np.isfinite(got).all(), f"call {call}: output not fully written"
        err = rel_err(got, ref)
        err_o = rel_err(got, ref_o)
        assert err <= UT_TOL and err_o <= UT_TOL, f"call {call}: rel err {err:.3e} (handle), {err_o:.3e} (oracle)"
        assert rel_err(ref, ref_o) <= UT_TOL
    # the second call (past the first-call set-up) left the device's free memory unchanged
    assert free[1][0] == free[1][1]
    del keep


def test_noalloc_rejects_oversized_mesh():
    """Host-side capacity check: fails before any CUDA call, with the reason in fg_last_error(NULL)."""
    L = _lib.load()
    c = make_config(N=7, NodeType="gauss-lobatto", SplitDG="pi")
    m = _lib.FgDeviceMesh(4096, 3 * 4096, 0, None, None, None, None, None, None, None)
    rc = L.fg_time_derivative_noalloc(ctypes.byref(c), ctypes.byref(m), None, None, None)
    assert rc == 1
    msg = L.fg_last_error(None).decode()
    assert "scratch" in msg and "maximum" in msg and str(_max_bytes()) in msg


def test_noalloc_rejects_unsupported_config():
    L = _lib.load()
    m = _lib.FgDeviceMesh(8, 24, 0, None, None, None, None, None, None, None)
    base = dict(N=3, NodeType="gauss", SplitDG="weak")
    for kw in (dict(doTCSource=1), dict(doWeakLifting=1), dict(N=5, NodeType="gauss-lobatto", SplitDG="pi"),
               dict(SplitDG="pi"), dict(N=9)):
        c = make_config(**{**base, **kw})
        rc = L.fg_time_derivative_noalloc(ctypes.byref(c), ctypes.byref(m), None, None, None)
        assert rc == 1 and "unsupported" in L.fg_last_error(None).decode()


def _max_bytes():
    import os
    import re

    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "flexi_gpu.h")).read()
    shift = int(re.search(r"#define FG_NOALLOC_SCRATCH_BYTES \(64ull << (\d+)\)", hdr).group(1))
    return 64 << shift
