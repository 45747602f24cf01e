"""Generates the golden fixtures under tests/golden/ from the reference's own test data.

Reads FLEXI v25.10's unit-test data (unitTests/*.bin, Fortran unformatted sequential records:
4-byte length marker, little-endian payload, closing marker) and the Taylor-Green regression
references (regressioncheck/checks/tgv/{split,splitGauss,oInt}/TGV_Re1600_*_TGVAnalysis_Reference.csv),
and stores the arrays the parity tests need in reference_unittests.npz, tgv_split_reference.npz,
tgv_splitgauss_reference.npz and tgv_oint_reference.npz; copies fifteen HOPR mesh / FLEXI state files
of the reference's test cases to hopr/ for the HDF5 reader.

Run from the repository root in a container that has the reference mounted:
    python tests/golden/make_golden.py <path of the FLEXI source tree>
"""
import os
import sys

import numpy as np


def read_records(path):
    """Fortran unformatted sequential file -> list of raw record payloads (bytes)."""
    data = open(path, "rb").read()
    recs, pos = [], 0
    while pos < len(data):
        n = int(np.frombuffer(data, dtype="<i4", count=1, offset=pos)[0])
        recs.append(data[pos + 4: pos + 4 + n])
        n2 = int(np.frombuffer(data, dtype="<i4", count=1, offset=pos + 4 + n)[0])
        assert n == n2, path
        pos += 8 + n
    return recs


def f64(buf, off, shape):
    cnt = int(np.prod(shape))
    return np.frombuffer(buf, dtype="<f8", count=cnt, offset=off).reshape(shape, order="F").copy(), off + 8 * cnt


def i32(buf, off, shape):
    cnt = int(np.prod(shape))
    return np.frombuffer(buf, dtype="<i4", count=cnt, offset=off).reshape(shape, order="F").copy(), off + 4 * cnt


def main(ref):
    ut = os.path.join(ref, "unitTests")
    out = {}
    NRef = 9
    n = NRef + 1
    # UnittestElementData3D.bin: nElems,SideToElem(5,6),firstMPISide_YOUR,lastMPISide_MINE,nSides,
    # S2V2(2,0:9,0:9,0:4,1:6),S2V(3,0:9,0:9,0:9,0:4,1:6),L_Minus,L_Plus,L_HatPlus,L_HatMinus,sJ(0:9,0:9,0:9,0:1,1)
    (rec,) = read_records(os.path.join(ut, "UnittestElementData3D.bin"))
    off = 0
    nElems, off = i32(rec, off, (1,))
    S2E, off = i32(rec, off, (5, 6))
    fMY, off = i32(rec, off, (1,))
    lMM, off = i32(rec, off, (1,))
    nSides, off = i32(rec, off, (1,))
    S2V2, off = i32(rec, off, (2, n, n, 5, 6))
    S2V, off = i32(rec, off, (3, n, n, n, 5, 6))
    Lm, off = f64(rec, off, (n,))
    Lp, off = f64(rec, off, (n,))
    LhP, off = f64(rec, off, (n,))
    LhM, off = f64(rec, off, (n,))
    sJ, off = f64(rec, off, (n, n, n, 2, 1))
    assert off == len(rec), (off, len(rec))
    out.update(elem_nElems=nElems, elem_SideToElem=S2E, elem_nSides=nSides, elem_S2V2=S2V2, elem_S2V=S2V,
               elem_L_Minus=Lm, elem_L_Plus=Lp, elem_L_HatPlus=LhP, elem_L_HatMinus=LhM, elem_sJ=sJ,
               elem_firstMPISide_YOUR=fMY, elem_lastMPISide_MINE=lMM)
    (rec,) = read_records(os.path.join(ut, "ProlongToFaceUvol.bin"))
    out["prolong_Uvol"], _ = f64(rec, 0, (n, n, n, 1))
    for tag in ("G3D", "GL3D"):
        recs = read_records(os.path.join(ut, f"ProlongToFace_{tag}.bin"))
        out[f"prolong_{tag}"], _ = f64(recs[0], 0, (n, n, 6))
    (rec,) = read_records(os.path.join(ut, "SurfIntFlux.bin"))
    out["surfint_Flux"], _ = f64(rec, 0, (n, n, 6))
    for tag in ("G3D", "GL3D", "G3D_Split"):
        recs = read_records(os.path.join(ut, f"SurfInt_{tag}.bin"))
        out[f"surfint_{tag}"], _ = f64(recs[0], 0, (n, n, n, 1))
    (rec,) = read_records(os.path.join(ut, "NodesAndWeights.bin"))
    xi, off = f64(rec, 0, (11, 10, 4))
    w, off = f64(rec, off, (11, 10, 4))
    wb, off = f64(rec, off, (11, 10, 4))
    out.update(nw_xi=xi, nw_w=w, nw_wBary=wb)
    (rec,) = read_records(os.path.join(ut, "DerivativeMatrix.bin"))
    out["dmat_D"], _ = f64(rec, 0, (11, 11, 40))
    np.savez_compressed(os.path.join(os.path.dirname(__file__), "reference_unittests.npz"), **out)

    # tgv/split (Gauss-Lobatto, N=7) and tgv/splitGauss (Gauss, N=5, entropy-variable prolongation)
    for case, name, fname in (("split", "tgv_split_reference.npz", "TGV_Re1600_Split_TGVAnalysis_Reference.csv"),
                              ("splitGauss", "tgv_splitgauss_reference.npz", "TGV_Re1600_Split_TGVAnalysis_Reference.csv"),
                              ("oInt", "tgv_oint_reference.npz", "TGV_Re1600_OInt_TGVAnalysis_Reference.csv")):
        csv = os.path.join(ref, f"regressioncheck/checks/tgv/{case}/{fname}")
        lines = open(csv).read().strip().splitlines()
        header = [h.strip() for h in lines[0].split(",")]
        rows = np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]])
        np.savez_compressed(os.path.join(os.path.dirname(__file__), name), header=np.array(header), rows=rows)
        print("wrote", name, rows.shape)
    # HOPR mesh and FLEXI state files of the reference's test cases, for the HDF5 reader and the mesh
    # read-in (copied unchanged)
    import shutil
    hdir = os.path.join(os.path.dirname(__file__), "hopr")
    os.makedirs(hdir, exist_ok=True)
    for src in ("regressioncheck/checks/tgv/oInt/CART_HEX_PERIODIC_004_mesh.h5", "tutorials/channel/CHANNEL_004_mesh.h5",
                "regressioncheck/checks/convtest/p_3D_mortar/CART_HEX_PERIODIC_MORTAR_002_mesh.h5",
                "regressioncheck/checks/timedisc/freestream_3D/cartbox3D_mesh.h5",
                "regressioncheck/checks/timedisc/freestream_3D/cartbox_State_0000000.000000000.h5",
                "tutorials/naca0012/NACA0012_652_Ng2_mesh.h5",
                "regressioncheck/checks/run_basic/freestream_3D/cartbox3D_mortar_mesh.h5") + tuple(
                f"regressioncheck/checks/convtest/h_3D_mortar/CART_HEX_PERIODIC_MORTAR_FLIPPED_{k:03d}_mesh.h5" for k in (1, 2, 4, 8)) + tuple(
                f"regressioncheck/checks/convtest/h_3D/CART_HEX_PERIODIC_{k:03d}_3D_mesh.h5" for k in (1, 2, 4, 8)):
        shutil.copyfile(os.path.join(ref, src), os.path.join(hdir, os.path.basename(src)))
    print("wrote fixtures:", sorted(out.keys()))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the FLEXI source tree>")
    main(sys.argv[1])
