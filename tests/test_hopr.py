"""HOPR mesh files through the library's HDF5 reader (fg_hopr_sizes / fg_hopr_read, flexi_gb300.mesh.read_hopr).

Fixtures: mesh and state files of the reference's own test cases (tests/golden/hopr/, copied by
tests/golden/make_golden.py). Checks: sizes, connectivity and BCs as mesh_readin.f90 interprets them;
the reference's periodic 4^3 TGV mesh gives the same operator as the synthetic box (the oracle's time
derivative agrees to round-off after matching elements by their barycentres); a fluid at rest between
isothermal walls of the reference's channel mesh is a steady state (Ut at round-off, which a wrongly
read wall would break), and likewise on the curved (NGeo=2) NACA0012 mesh, whose free-stream preservation
needs the curved metrics built from the file's nodes; BC overrides by name; truncated and non-HDF5 files
give errors.
"""
import os
import shutil

import numpy as np
import pytest

from _cases import perturb_state
from flexi_gb300 import mesh as fmesh, testcases
from oracle import oracle as orc

HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")
CFG = dict(N=3, nodeType=orc.NT_GAUSS, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=-1,
           etaBR2=2.0, etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=6.25e-4, CFLScale=0.9, DFLScale=0.9,
           doTCSource=0, dpdx=-1.0)


def _path(name):
    return os.path.join(HOPR, name)


def test_periodic_box_connectivity():
    m = fmesh.read_hopr(_path("CART_HEX_PERIODIC_004_mesh.h5"))
    assert m.n_elems == 64 and m.ngeo == 1
    assert len(m.bc_names) == 6 and (m.boundary_type[:, 0] == 1).all()  # all periodic
    assert (m.elem_nb[:, :, 0] > 0).all() and (m.elem_nb[:, :, 2] == 0).all()
    # symmetric connections: my neighbour's side points back at me
    for e in range(m.n_elems):
        for ls in range(6):
            ne, nls, _ = m.elem_nb[e, ls]
            assert m.elem_nb[ne - 1, nls - 1, 0] == e + 1 and m.elem_nb[ne - 1, nls - 1, 1] == ls + 1
    assert np.allclose(m.node_coords.min(axis=(0, 1, 2, 3)), 0.0) and np.allclose(m.node_coords.max(axis=(0, 1, 2, 3)), 2 * np.pi)


def _barycentres(m):
    return m.node_coords.reshape(m.n_elems, -1, 3).mean(axis=1)


def test_periodic_box_operator_matches_synthetic_box():
    """The file's box is [0, 2 pi]^3, the synthetic one [-pi, pi]^3: in a periodic box the shift by pi keeps
    every neighbour relation, so element e of the file corresponds to the synthetic element at its
    barycentre minus pi, with the same nodal state."""
    mh = fmesh.read_hopr(_path("CART_HEX_PERIODIC_004_mesh.h5"))
    ms = fmesh.tgv_box(4, ngeo=1)
    bh, bs = _barycentres(mh) - np.pi, _barycentres(ms)
    perm = np.array([int(np.argmin(np.linalg.norm(bs - b, axis=1))) for b in bh])  # synthetic index of each file element
    assert np.allclose(bs[perm], bh, atol=1e-12) and len(set(perm.tolist())) == mh.n_elems
    oh, os_ = orc.Oracle(CFG, mh), orc.Oracle(CFG, ms)
    xh = oh.mesh_array("Elem_xGP")
    assert np.allclose(xh - np.pi, os_.mesh_array("Elem_xGP")[perm], atol=1e-12)
    U = perturb_state(testcases.tgv_state(xh, mach=0.1, kappa=1.4, R=71.42857), seed=2)
    Us = np.empty_like(U)
    Us[perm] = U
    oh.set_state(U)
    os_.set_state(Us)
    uh, us = oh.time_derivative(0.0), os_.time_derivative(0.0)[perm]
    assert np.abs(uh - us).max() <= 1e-12 * np.abs(us).max()


def test_channel_walls_at_rest_are_steady():
    T = 1.0
    p = 1.0
    rho = p / (71.42857 * T)
    m = fmesh.read_hopr(_path("CHANNEL_004_mesh.h5"), ref_state_prim=[[rho, 0.0, 0.0, 0.0, p, T]])
    assert sorted(m.bc_names) == sorted(["BC_periodicz-", "BC_wall_lower", "BC_periodicx+", "BC_wall_upper", "BC_periodicx-",
                                         "BC_periodicz+"])
    walls = [i + 1 for i, nm in enumerate(m.bc_names) if "wall" in nm]
    assert all(tuple(m.boundary_type[w - 1]) == (4, 1) for w in walls)
    n_wall = int(np.isin(m.elem_nb[:, :, 2], walls).sum())
    assert n_wall == 2 * 4 * 4 and (m.elem_nb[:, :, 0] == 0).sum() == n_wall
    o = orc.Oracle(dict(CFG, riemann=3), m)
    x = o.mesh_array("Elem_xGP")
    U = np.zeros(x.shape[:-1] + (5,))
    U[..., 0] = rho
    U[..., 4] = p / 0.4
    o.set_state(U)
    assert np.abs(o.time_derivative(0.0)).max() <= 1e-11


def test_boundary_override_by_name():
    m = fmesh.read_hopr(_path("cartbox3D_mesh.h5"))
    assert (m.boundary_type[:, 0] == 2).all()  # Dirichlet in the file
    m2 = fmesh.read_hopr(_path("cartbox3D_mesh.h5"), boundary={nm: (3, 0) for nm in m.bc_names})
    assert (m2.boundary_type == [3, 0]).all()
    with pytest.raises(KeyError):
        fmesh.read_hopr(_path("cartbox3D_mesh.h5"), boundary={"BC_nonexistent": (3, 0)})


def test_unsupported_and_corrupt_files(tmp_path):
    mo = fmesh.read_hopr(_path("CART_HEX_PERIODIC_MORTAR_002_mesh.h5"))  # mortar meshes read (tables checked in test_oracle_mortar)
    assert mo.n_elems == 28 and len(mo.mortars) == 8
    data = open(_path("CART_HEX_PERIODIC_004_mesh.h5"), "rb").read()
    for cut in (64, 2000, len(data) // 2):
        p = tmp_path / f"cut{cut}.h5"
        p.write_bytes(data[:cut])
        with pytest.raises(ValueError):
            fmesh.read_hopr(p)
    p = tmp_path / "text.h5"
    p.write_text("not an HDF5 file\n" * 100)
    with pytest.raises(ValueError, match="not an HDF5 file"):
        fmesh.read_hopr(p)
    with pytest.raises(ValueError, match="Ngeo"):  # a state file is no mesh
        fmesh.read_hopr(_path("cartbox_State_0000000.000000000.h5"))
    p = tmp_path / "copy.h5"
    shutil.copyfile(_path("CART_HEX_PERIODIC_004_mesh.h5"), p)
    assert fmesh.read_hopr(p).n_elems == 64


def test_curved_airfoil_mesh_at_rest_is_steady():
    """NACA0012, 652 curved elements (NGeo=2), inflow/outflow replaced by adiabatic walls: a fluid at rest is
    steady to round-off (|Ut| against O(100) for a moving fluid)."""
    m = fmesh.read_hopr(_path("NACA0012_652_Ng2_mesh.h5"), boundary={"BC_inflow": (3, 0), "BC_outflow": (3, 0)})
    assert m.n_elems == 652 and m.ngeo == 2
    o = orc.Oracle(dict(CFG, riemann=3, R=1.0, mu0=1e-3), m)
    x = o.mesh_array("Elem_xGP")
    U = np.zeros(x.shape[:-1] + (5,))
    U[..., 0] = 1.0
    U[..., 4] = 1.0 / 0.4
    o.set_state(U)
    assert np.abs(o.time_derivative(0.0)).max() <= 1e-10
    U[..., 1] = 0.3
    o.set_state(U)
    assert np.abs(o.time_derivative(0.0)).max() > 1.0
