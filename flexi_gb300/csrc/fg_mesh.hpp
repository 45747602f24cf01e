// flexi_gb300 -- host-side mesh preparation: everything FLEXI's InitMesh provides to the DG operator
// (src/mesh/mesh.f90:InitMesh, prepare_mesh.f90, mappings.f90, metrics.f90:CalcMetrics/CalcSurfMetrics),
// produced directly in the device layouts used by the kernels:
//   metr [e][9][n3]  Metrics_fTilde(3), Metrics_gTilde(3), Metrics_hTilde(3) per volume node
//   sJ   [e][n3]     inverse Jacobian
//   geo  [s][10][n2] NormVec(3), TangVec1(3), TangVec2(3), SurfElem per side point (master orientation)
//   faceJa [e][6][3][n2] normal-direction row of each element's own face metrics (split form, Gauss nodes)
// Two entry points: from raw element node coordinates and element connectivity (the content of a HOPR
// mesh file: NodeCoords on equidistant NGeo points, neighbour ids), or from the arrays FLEXI itself has
// built (the drop-in path, where FLEXI keeps doing its own InitMesh and hands the result over).
#pragma once
#include "fg_basis.hpp"
#include <string>

namespace fgh {

struct RawMesh {
  int nElems = 0, NGeo = 1;
  const double* nodeCoords = nullptr;  // Fortran (3,0:NGeo,0:NGeo,0:NGeo,nElems)
  const int* elemNb = nullptr;         // (3,6,nElems): neighbour elem (1-based, 0 = boundary), neighbour local side, BC index
  int nBCs = 0;
  const int* boundaryType = nullptr;   // (2,nBCs): BC type, BC state
  int nRefStates = 0;
  const double* refStatePrim = nullptr;  // (6,nRefStates)
  const int* elemInst = nullptr;       // optional instance id per element (ensembles)
  // mortar interfaces (elemNb neighbour -1), 15 per mortar: big element (1-based), its local side, type
  // (1: 1->4, 2: 1->2 in eta, 3: 1->2 in xi), then per small side: element (1-based), local side, unused
  int nMortars = 0;
  const int* mortars = nullptr;
};

struct HostMesh {
  int N = 0, n = 0, nodeType = 2, nElems = 0, nSides = 0, nBCSides = 0;
  // sides are ordered BC | conforming inner | small mortar | big mortar; nFluxSides = BC + conforming inner
  int nFluxSides = 0, nMortars = 0;
  std::vector<int> mortarInfo;  // [m][6]: type, big side, small sides (-1: unused)
  std::vector<int> flexiSide;   // drop-in meshes: FLEXI's SideID - 1 of each side (empty: identity)
  std::vector<int> sideElem;    // [s][4]
  std::vector<int> elemSide;    // [e][6]
  std::vector<int> sideInst, elemInst;
  std::vector<int> bcType;      // [nBCSides]
  std::vector<double> bcTwall;  // [nBCSides]
  std::vector<double> metr, sJ, geo;
  // [e][6][3][n2]: row NormalDir of the element's own face metrics on each of its sides (Ja_Face for the
  // master, Ja_slave for the slave side, metrics.f90:CalcSurfMetrics), indexed by the element's face
  // coordinates (a + n*b); used by the split form on Gauss nodes
  std::vector<double> faceJa;
  std::vector<double> elemX;    // [e][3][n3] solution point coordinates (Elem_xGP)
  std::vector<double> wVol;     // [n3] tensor-product quadrature weights
  std::vector<double> metAdv, metVisc;  // [e][3][n3] calctimestep.f90:InitCalctimestep
  std::vector<double> instVol;  // per instance domain volume
  int nInst = 1;
};

// builds sides, orientation flips and metrics from node coordinates and connectivity
void build_from_raw(const RawMesh& raw, int N, int nodeType, HostMesh& M);
// takes FLEXI's own processed mesh arrays (Fortran layouts, 1-based ids)
void build_from_flexi(int N, int nodeType, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide,
                      const int* BC, int nBCs, const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Mf,
                      const double* Mg, const double* Mh, const double* sJ, const double* NormVec, const double* TangVec1,
                      const double* TangVec2, const double* SurfElem, int nMortars, const int* MortarType, const int* MortarInfo,
                      HostMesh& M);
// derived per-node quantities (time-step metrics, quadrature weights, instance volumes)
void finish_mesh(HostMesh& M, double kappa, double Pr);

}  // namespace fgh
