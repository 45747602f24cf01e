"""CPU tests of the product library's host side: C ABI exports, configuration, ini parsing, and the
mesh preparation (sides, flips, curl-form metrics, surface metrics) against the oracle's restatement
of FLEXI's InitMesh/CalcMetrics. No GPU work is issued here."""
import ctypes
import dataclasses
import os
import re

import numpy as np
import pytest

from flexi_gb300 import _lib, mesh as fmesh
from flexi_gb300.solver import Flexi, FlexiError, make_config, config_from_ini, config_dict
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from flexi_gb300 import build
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    header = open(os.path.join(ROOT, "include", "flexi_gpu.h")).read()
    declared = set(re.findall(r"^\s*(?:int|const char\*|long long)\s+(fg_\w+)\s*\(", header, re.M))
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(_lib.EXPORTS)


def test_config_defaults_and_validation(lib):
    c = make_config()
    d = config_dict(c)
    assert d["Riemann"] == 33 and d["SplitDG"] == 4 and d["Lifting"] == 1 and d["kappa"] == 1.4 and d["R"] == 287.058
    assert d["CFLScale"] == 0.9 and d["etaBR2"] == 2.0 and d["Pr"] == 0.72
    with pytest.raises(FlexiError):
        Flexi(make_config(N=12))
    with pytest.raises(FlexiError):
        Flexi(make_config(N=5, SplitDG=7))  # splitflux.f90:63-69 defines SplitDG 0..6
    with pytest.raises(FlexiError):
        Flexi(make_config(N=5, SplitDG="weak", Riemann="ch"))  # CH, IR and avg need the split form
    with pytest.raises(FlexiError):
        Flexi(make_config(N=5, Riemann=9))  # no solver 9 in riemann.f90:44-58
    with pytest.raises(FlexiError):
        Flexi(make_config(N=5, OverintegrationType=3))
    # lifting.f90:137-139: BR2 lifts in strong form, doWeakLifting is dropped; doConservativeLifting stays
    f = Flexi(make_config(N=3, Lifting="br2", doWeakLifting=1, doConservativeLifting=1))
    d = config_dict(f.get_config())
    assert d["doWeakLifting"] == 0 and d["doConservativeLifting"] == 1
    f.close()


def test_ini_parser(lib):
    # keys as written in regressioncheck/checks/tgv/split/parameter.ini
    text = """
    N             = 7 ! Polynomial degree
    Riemann               =  RoeEntropyFix ! Riemann solver
    SplitDG               = PI
    Mu0           = 6.25E-04    ! viscosity set to 1/Re
    R             = 71.42857
    CFLscale   = 0.8  ! Scaling of theoretical CFL number
    DFLscale   = 0.8
    NodeType = Gauss-Lobatto
    Lifting = br2
    etaBR2 = 3.
    """
    d = config_dict(config_from_ini(text))
    assert d["N"] == 7 and d["Riemann"] == 33 and d["SplitDG"] == 4 and d["mu0"] == 6.25e-4 and d["R"] == 71.42857
    assert d["CFLScale"] == 0.8 and d["DFLScale"] == 0.8 and d["NodeType"] == 2 and d["Lifting"] == 2 and d["etaBR2"] == 3.0


def _oracle_cfg(N, node_type):
    return dict(N=N, nodeType=node_type, riemann=33, riemannBC=-1, lifting=1, weakLifting=0, consLifting=0, splitDG=-1, etaBR2=2.0,
                etaBR2_wall=-1.0, kappa=1.4, R=71.42857, Pr=0.72, mu0=1e-3, CFLScale=0.9, DFLScale=0.9, doTCSource=0, dpdx=-1.0)


MESHES = {
    "cartesian": lambda: fmesh.tgv_box(3, ngeo=1),
    "curved": lambda: fmesh.tgv_box(3, ngeo=3, perturb=0.3, seed=1),
    "channel": lambda: fmesh.channel_box((3, 4, 2), beta=1.5, ngeo=2),
}


@pytest.mark.parametrize("mesh_name", list(MESHES))
@pytest.mark.parametrize("N,node_type", [(3, 1), (4, 2), (7, 2)])
def test_mesh_preparation_matches_oracle(lib, mesh_name, N, node_type):
    m = MESHES[mesh_name]()
    o = orc.Oracle(_oracle_cfg(N, node_type), m)
    f = Flexi(make_config(N=N, NodeType=node_type, SplitDG=-1))
    f.build_mesh(m, host_only_ok=True)
    assert (f.n_elems, f.n_sides, f.n_bc_sides) == (o.n_elems, o.n_sides, o.n_bc_sides)
    assert np.array_equal(f.side_to_elem(), o.mesh_iarray("SideToElem"))
    for name in ("Mf", "Mg", "Mh"):
        a, b = f.mesh_array(name), o.mesh_array(name)
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max()), name
    assert np.abs(f.mesh_array("sJ") / o.mesh_array("sJ") - 1).max() < 1e-13
    np.testing.assert_allclose(f.elem_xgp(), o.mesh_array("Elem_xGP"), rtol=0, atol=1e-13)
    # face metrics: master sides are stored by both in the same side numbering
    for name in ("NormVec", "TangVec1", "TangVec2", "SurfElem"):
        a, b = f.mesh_array(name), o.mesh_array(name)
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max()), name
    f.close()


HOPR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hopr")


def _side_keys(s2e):
    """side -> (slave element, slave local side) where there is a slave, else (master element, its local side)"""
    return [("s", int(r[1]), int(r[3])) if r[1] > 0 else ("m", int(r[0]), int(r[2])) for r in s2e]


@pytest.mark.parametrize("mesh_file", ["CART_HEX_PERIODIC_MORTAR_002_mesh.h5", "CART_HEX_PERIODIC_MORTAR_FLIPPED_002_mesh.h5",
                                       "cartbox3D_mortar_mesh.h5"])
@pytest.mark.parametrize("N,node_type", [(3, 1), (4, 2)])
def test_mortar_mesh_preparation_matches_oracle(lib, mesh_file, N, node_type):
    """Mortar sides (mesh_readin.f90 MortarType/MortarInfo, mortar_metrics.f90:Mortar_CalcSurfMetrics): the
    library orders sides BC | conforming | small | big, the oracle BC | big | conforming | small; matched by
    (slave element, its local side), or (master element, its local side) for sides without a slave, every
    side has the same flip and the same normals, tangents and surface elements. Small sides carry the big
    element as master in the library (its viscosity), none in the oracle."""
    m0 = fmesh.read_hopr(os.path.join(HOPR, mesh_file))
    m = fmesh.read_hopr(os.path.join(HOPR, mesh_file), boundary={nm: (3, 0) for nm in m0.bc_names if nm != "inner"})
    o = orc.Oracle(_oracle_cfg(N, node_type), m)
    f = Flexi(make_config(N=N, NodeType=node_type, SplitDG=-1))
    f.build_mesh(m, host_only_ok=True)
    assert (f.n_elems, f.n_sides, f.n_bc_sides) == (o.n_elems, o.n_sides, o.n_bc_sides)
    fs, os_ = f.side_to_elem(), o.mesh_iarray("SideToElem")
    ko = {k: i for i, k in enumerate(_side_keys(os_))}
    perm = np.array([ko[k] for k in _side_keys(fs)])
    assert len(set(perm.tolist())) == f.n_sides
    assert np.array_equal(fs[:, [1, 3, 4]], os_[perm][:, [1, 3, 4]])  # slave, its local side, flip
    small = os_[perm, 0] == -1
    assert small.sum() == sum(4 if t == 1 else 2 for t in m.mortars[:, 2])
    assert np.array_equal(fs[~small][:, [0, 2]], os_[perm[~small]][:, [0, 2]])
    for name in ("NormVec", "TangVec1", "TangVec2", "SurfElem"):
        a, b = f.mesh_array(name), o.mesh_array(name)[perm]
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max()), name
    f.close()


def test_mortar_mesh_errors(lib):
    m = fmesh.read_hopr(os.path.join(HOPR, "CART_HEX_PERIODIC_MORTAR_002_mesh.h5"))
    f = Flexi(make_config(N=3, NodeType=1, SplitDG=-1))
    bad = dataclasses.replace(m, mortars=m.mortars[:-1])
    with pytest.raises(FlexiError, match="do not match the Mortars table"):
        f.build_mesh(bad, host_only_ok=True)
    swapped = m.mortars.copy()
    swapped[0, 3] = swapped[1, 3]  # a small side named twice
    with pytest.raises(FlexiError, match="mortar"):
        f.build_mesh(dataclasses.replace(m, mortars=swapped), host_only_ok=True)
    f.close()


def test_drop_in_mortar_mesh_tables(lib):
    """fg_set_mesh_mortar takes FLEXI's arrays (here the oracle's): the library's side tables equal those it
    builds itself from the mesh file (matched by slave / master element side), with the same geometry."""
    m = fmesh.read_hopr(os.path.join(HOPR, "CART_HEX_PERIODIC_MORTAR_002_mesh.h5"))
    o = orc.Oracle(_oracle_cfg(3, 1), m)
    arrays = [o.mesh_array(k) for k in ("Mf", "Mg", "Mh", "sJ", "NormVec", "TangVec1", "TangVec2", "SurfElem")]
    f = Flexi(make_config(N=3, NodeType=1, SplitDG=-1))
    f.set_mesh(o.mesh_iarray("SideToElem"), o.mesh_iarray("ElemToSide"), o.mesh_iarray("BC"), m.boundary_type, m.ref_state_prim,
               *arrays, mortar_type=o.mesh_iarray("MortarType"), mortar_info=o.mesh_iarray("MortarInfo"), host_only_ok=True)
    g = Flexi(make_config(N=3, NodeType=1, SplitDG=-1))
    g.build_mesh(m, host_only_ok=True)
    fs, gs = f.side_to_elem(), g.side_to_elem()
    kg = {k: i for i, k in enumerate(_side_keys(gs))}
    perm = np.array([kg[k] for k in _side_keys(fs)])
    assert np.array_equal(fs, gs[perm])
    for name in ("NormVec", "SurfElem"):
        a, b = f.mesh_array(name), g.mesh_array(name)[perm]
        assert np.abs(a - b).max() <= 1e-13 * max(1.0, np.abs(b).max()), name
    bad = o.mesh_iarray("MortarInfo").copy()
    bad[0, 0, 0] = bad[1, 0, 0]
    with pytest.raises(FlexiError, match="MortarInfo"):
        f.set_mesh(o.mesh_iarray("SideToElem"), o.mesh_iarray("ElemToSide"), o.mesh_iarray("BC"), m.boundary_type, m.ref_state_prim,
                   *arrays, mortar_type=o.mesh_iarray("MortarType"), mortar_info=bad, host_only_ok=True)
    f.close()
    g.close()


def test_ini_exact_function_keys(lib):
    # keys as written in regressioncheck/checks/convtest/h_3D_mortar/parameter.ini
    text = """
    IniExactFunc     = 4
    AdvVel           = (/0.3,0.2,0.1/)
    IniFrequency = 2.0
    IniAmplitude = 0.05
    """
    d = config_dict(config_from_ini(text))
    assert d["IniExactFunc"] == 4 and d["AdvVel"] == (0.3, 0.2, 0.1) and d["IniFrequency"] == 2.0 and d["IniAmplitude"] == 0.05
    d0 = config_dict(make_config())
    assert d0["IniExactFunc"] == 0 and d0["IniFrequency"] == 1.0 and d0["IniAmplitude"] == 0.1 and d0["AdvVel"] == (0.0, 0.0, 0.0)
    assert config_dict(make_config(AdvVel=(1.0, 2.0, 3.0)))["AdvVel"] == (1.0, 2.0, 3.0)
    with pytest.raises(FlexiError):
        config_from_ini("AdvVel = (/0.3,0.2/)\n")


def test_ensemble_of_mortar_instances(lib):
    """concatenate() keeps mortar sides (-1) and offsets the Mortars table: an ensemble of a mortar box and a
    plain box prepares the same sides as the two meshes separately."""
    a, b = fmesh.mortar_box(2, perturb=0.05, seed=1), fmesh.tgv_box(2)
    e = fmesh.concatenate([a, b])
    assert len(e.mortars) == len(a.mortars) and (e.elem_nb[:, :, 0] == -1).sum() == (a.elem_nb[:, :, 0] == -1).sum()
    fe = Flexi(make_config(N=3, NodeType=1, SplitDG=-1))
    fe.build_mesh(e, host_only_ok=True)
    sizes = []
    for m in (a, b):
        f = Flexi(make_config(N=3, NodeType=1, SplitDG=-1))
        f.build_mesh(m, host_only_ok=True)
        sizes.append(f.n_sides)
        f.close()
    assert fe.n_sides == sum(sizes)
    fe.close()
