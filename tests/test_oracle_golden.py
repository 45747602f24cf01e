"""Pins the CPU oracle to FLEXI's own golden data (unitTests/*.bin, regressioncheck TGV CSV).

Tolerances are those of the reference's unit tests: ALMOSTEQUALABSORREL with 50/100 x PP_RealTolerance
(unitTests/NodesAndWeights.f90, DerivativeMatrix.f90, ProlongToFace.f90, SurfInt.f90).
"""
import numpy as np
import pytest

from oracle import oracle as orc

EPS = np.finfo(np.float64).eps


def almost_equal_abs_or_rel(a, b, tol):
    # globals.f90:ALMOSTEQUALABSORREL -- |a-b| <= max(tol, tol*|b|)
    return np.abs(a - b) <= np.maximum(tol, tol * np.abs(b))


def test_nodes_and_weights(golden):
    xi_ref, w_ref, wb_ref = golden["nw_xi"], golden["nw_w"], golden["nw_wBary"]
    for t, nt in enumerate((orc.NT_GAUSS, orc.NT_GL, orc.NT_CL, orc.NT_VISU)):
        for N in range(1, 11):
            x, w, wb = orc.nodes_and_weights(N, nt)
            assert almost_equal_abs_or_rel(x, xi_ref[: N + 1, N - 1, t], 50 * EPS).all(), (nt, N)
            assert almost_equal_abs_or_rel(w, w_ref[: N + 1, N - 1, t], 50 * EPS).all(), (nt, N)
            assert almost_equal_abs_or_rel(wb, wb_ref[: N + 1, N - 1, t], 50 * EPS).all(), (nt, N)


def test_derivative_matrix(golden):
    D_ref = golden["dmat_D"]
    for t, nt in enumerate((orc.NT_GAUSS, orc.NT_GL, orc.NT_CL, orc.NT_VISU)):
        for N in range(1, 11):
            D = orc.derivative_matrix(N, nt)
            ref = D_ref[: N + 1, : N + 1, t * 10 + N - 1]
            assert almost_equal_abs_or_rel(D, ref, 100 * EPS).all(), (nt, N)


def test_mappings_match_reference_tables(golden):
    # S2V2(2,0:N,0:N,0:4,1:6) and S2V(3,0:N,0:N,0:N,0:4,1:6) from UnittestElementData3D.bin (NRef=9)
    S2V2, S2V = orc.mappings(9)
    ref2 = golden["elem_S2V2"]  # Fortran (2,10,10,5,6)
    ref3 = golden["elem_S2V"]   # Fortran (3,10,10,10,5,6)
    assert np.array_equal(S2V2, np.transpose(ref2, (4, 3, 2, 1, 0)))
    assert np.array_equal(S2V, np.transpose(ref3, (5, 4, 3, 2, 1, 0)))


@pytest.mark.parametrize("tag,node_type", [("G3D", orc.NT_GAUSS), ("GL3D", orc.NT_GL)])
def test_prolong_to_face(golden, tag, node_type):
    N = 9
    s2e = golden["elem_SideToElem"].T.copy()
    s2v2 = np.transpose(golden["elem_S2V2"], (4, 3, 2, 1, 0)).copy()
    Uvol = np.transpose(golden["prolong_Uvol"][..., 0], (2, 1, 0)).copy()
    Um = orc.prolong_unittest(N, node_type, s2e, s2v2, golden["elem_L_Minus"], golden["elem_L_Plus"], Uvol)
    ref = np.transpose(golden[f"prolong_{tag}"], (2, 1, 0))
    assert almost_equal_abs_or_rel(Um, ref, 100 * EPS).all()


@pytest.mark.parametrize("tag,node_type", [("G3D", orc.NT_GAUSS), ("GL3D", orc.NT_GL)])
def test_surf_int(golden, tag, node_type):
    N = 9
    s2e = golden["elem_SideToElem"].T.copy()
    s2v2 = np.transpose(golden["elem_S2V2"], (4, 3, 2, 1, 0)).copy()
    flux = np.transpose(golden["surfint_Flux"], (2, 1, 0)).copy()
    Ut = orc.surfint_unittest(N, node_type, s2e, s2v2, golden["elem_L_HatMinus"], golden["elem_L_HatPlus"], flux)
    ref = np.transpose(golden[f"surfint_{tag}"][..., 0], (2, 1, 0))
    assert almost_equal_abs_or_rel(Ut, ref, 100 * EPS).all()


def test_surf_int_split_gauss(golden):
    """unitTests/SurfInt.f90 with SPLIT_DG on Gauss nodes: the split-Gauss surface integral of a random flux
    with unit states and metrics (its correction vanishes for a constant state); the reference compares at
    200 x PP_RealTolerance."""
    N = 9
    s2e = golden["elem_SideToElem"].T.copy()
    flux = np.transpose(golden["surfint_Flux"], (2, 1, 0)).copy()
    Ut = orc.surfint_split_unittest(N, s2e, golden["elem_L_Minus"], golden["elem_L_Plus"], golden["elem_L_HatMinus"],
                                    golden["elem_L_HatPlus"], flux)
    ref = np.transpose(golden["surfint_G3D_Split"][..., 0], (2, 1, 0))
    assert almost_equal_abs_or_rel(Ut, ref, 200 * EPS).all()
