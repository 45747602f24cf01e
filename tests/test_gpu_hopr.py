"""GPU path on HOPR mesh files and FLEXI state files (mesh_readin.f90, hdf5_output.f90:WriteState, restart).

- Ut on the reference's periodic TGV mesh, channel mesh (isothermal walls) and curved NACA0012 mesh
  (NGeo=2, adiabatic walls) against the oracle on the same file, 1e-12 as in test_gpu_parity.py; a fluid
  at rest on the curved mesh stays at rest on the GPU too.
- fg_write_state / fg_read_state: a written state reads back bit for bit with its Time; a state of another
  N is refused; the reference's own freestream state file (tests/golden/hopr/, N=3 Gauss) reads as the
  constant state (1, 1, 1, 1, 4) it holds.
"""
import os

import numpy as np
import pytest

from _cases import oracle_cfg, perturb_state, product_cfg, rel_err
from flexi_gb300 import mesh as fmesh, testcases
from flexi_gb300.solver import Flexi, FlexiError
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
COMMON = dict(kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4)


def _pair(c, m, U0):
    f = Flexi(c, m)
    o = orc.Oracle(oracle_cfg(c), m)
    f.U = U0
    o.set_state(U0)
    return f, o


@pytest.mark.parametrize("kw", [dict(N=5, NodeType="gauss", SplitDG="weak", Riemann="roeentropyfix"),
                                dict(N=7, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roeentropyfix", Lifting="br2")])
def test_rhs_parity_periodic_box_file(kw):
    c = product_cfg(**kw, **COMMON)
    m = fmesh.read_hopr(os.path.join(HOPR, "CART_HEX_PERIODIC_004_mesh.h5"))
    f = Flexi(c, m)
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.1, kappa=1.4, R=71.42857), seed=9)
    f.close()
    f, o = _pair(c, m, U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


def test_rhs_parity_channel_file():
    T, p = 1.0, 1.0
    rho = p / (1.0 * T)
    c = product_cfg(N=5, NodeType="gauss", SplitDG="weak", Riemann="roe", Lifting="br1", kappa=1.4, R=1.0, Pr=0.72, mu0=1e-3)
    m = fmesh.read_hopr(os.path.join(HOPR, "CHANNEL_004_mesh.h5"), ref_state_prim=[[rho, 0.0, 0.0, 0.0, p, T]])
    f = Flexi(c, m)
    U0 = testcases.channel_state(f.elem_xgp(), mach=0.3, kappa=1.4, R=1.0, t_wall=T, noise=0.05, seed=3)
    f.close()
    f, o = _pair(c, m, U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err


def test_state_file_round_trip(tmp_path):
    c = product_cfg(N=4, NodeType="gauss-lobatto", SplitDG="weak", Riemann="roe", **COMMON)
    m = fmesh.tgv_box(3, ngeo=2, perturb=0.1, seed=1)
    f = Flexi(c, m)
    U0 = perturb_state(testcases.tgv_state(f.elem_xgp(), mach=0.2, kappa=1.4, R=71.42857), seed=4)
    f.U = U0
    path = tmp_path / "tgv_State_0000000.250000000.h5"
    f.write_state(path, project="tgv", mesh_file="tgv_mesh.h5", t=0.25)
    g = Flexi(c, m)
    assert g.read_state(path) == 0.25
    assert np.array_equal(g.U, U0)
    c6 = product_cfg(N=5, NodeType="gauss-lobatto", SplitDG="weak", Riemann="roe", **COMMON)
    h = Flexi(c6, m)
    with pytest.raises(FlexiError, match="N = 4"):
        h.read_state(path)
    for x in (f, g, h):
        x.close()


def test_reads_reference_state_file():
    c = product_cfg(N=3, NodeType="gauss", SplitDG="weak", Riemann="roe", kappa=1.4, R=1.0, Pr=0.72, mu0=1.8547e-5)
    m0 = fmesh.read_hopr(os.path.join(HOPR, "cartbox3D_mesh.h5"))
    m = fmesh.read_hopr(os.path.join(HOPR, "cartbox3D_mesh.h5"), boundary={nm: (3, 0) for nm in m0.bc_names})
    f = Flexi(c, m)
    t = f.read_state(os.path.join(HOPR, "cartbox_State_0000000.000000000.h5"))
    U = f.U
    f.close()
    assert t == 0.0
    assert np.array_equal(U, np.broadcast_to(np.array([1.0, 1.0, 1.0, 1.0, 4.0]), U.shape))


def test_curved_airfoil_file():
    c = product_cfg(N=4, NodeType="gauss-lobatto", SplitDG="pi", Riemann="roe", Lifting="br2", kappa=1.4, R=1.0, Pr=0.72, mu0=1e-3)
    m = fmesh.read_hopr(os.path.join(HOPR, "NACA0012_652_Ng2_mesh.h5"), boundary={"BC_inflow": (3, 0), "BC_outflow": (3, 0)})
    f = Flexi(c, m)
    x = f.elem_xgp()
    rest = np.zeros(x.shape[:-1] + (5,))
    rest[..., 0] = 1.0
    rest[..., 4] = 1.0 / 0.4
    f.U = rest
    assert np.abs(f.DGTimeDerivative_weakForm(0.0)).max() <= 1e-10
    rng = np.random.default_rng(5)
    U0 = rest.copy()
    U0[..., 1] = 0.2 * np.sin(x[..., 0]) + 0.02 * rng.standard_normal(x.shape[:-1])
    U0[..., 2] = 0.1 * np.cos(x[..., 1])
    U0[..., 4] += 0.5 * (U0[..., 1] ** 2 + U0[..., 2] ** 2)
    f.close()
    f, o = _pair(c, m, U0)
    err = rel_err(f.DGTimeDerivative_weakForm(0.0), o.time_derivative(0.0))
    f.close()
    assert err <= 1e-12, err
