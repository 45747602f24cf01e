// flexi_gb300 -- file I/O of the C ABI: HOPR mesh files (mesh_readin.f90:ReadMesh, the file part) and FLEXI
// state files (hdf5_output.f90:WriteState / restart.f90 read-in of DG_Solution), on the HDF5 subset of
// fg_h5.hpp. Host code only; the solver state goes through the public fg_get_state / fg_set_state.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <ctime>
#include <map>
#include <string>
#include <vector>

#include "../../include/flexi_gpu.h"
#include "fg_h5.hpp"

namespace {

thread_local std::string g_ioerr;

int io_fail(int code, const std::string& msg) {
  g_ioerr = msg;
  return code;
}

// HOPR element types FLEXI accepts for hexahedra: 108 (trilinear), 118 (non-planar), 208 (curved)
bool is_hexa(long long t) { return t == 108 || t == 118 || t == 208; }

struct Hopr {
  long long nElems = 0, NGeo = 1, nBCs = 0;
  std::vector<long long> elemInfo, sideInfo, bcType;
  std::vector<double> nodes;
  std::vector<std::string> bcNames;
};

// reads and checks the datasets ReadMesh / ReadBCs use (mesh_readin.f90:125-182, 197-500)
Hopr read_hopr(const char* path) {
  fgh5::Reader r(path);
  Hopr h;
  if (!r.attr_int("Ngeo", h.NGeo)) throw std::runtime_error(std::string(path) + ": no attribute Ngeo (not a HOPR mesh file)");
  std::vector<uint64_t> de, ds, dn, db;
  h.elemInfo = r.read_int("ElemInfo", &de);
  if (de.size() != 2 || de[1] != 6) throw std::runtime_error("ElemInfo must be (nElems, 6)");
  h.nElems = (long long)de[0];
  h.sideInfo = r.read_int("SideInfo", &ds);
  if (ds.size() != 2 || ds[1] != 5) throw std::runtime_error("SideInfo must be (nSides, 5)");
  h.nodes = r.read_real("NodeCoords", &dn);
  if (dn.size() != 2 || dn[1] != 3) throw std::runtime_error("NodeCoords must be (nNodes, 3)");
  h.bcType = r.read_int("BCType", &db);
  if (db.size() != 2 || db[1] != 4) throw std::runtime_error("BCType must be (nBCs, 4)");
  h.nBCs = (long long)db[0];
  h.bcNames = r.read_str("BCNames");
  if ((long long)h.bcNames.size() != h.nBCs) throw std::runtime_error("BCNames and BCType differ in length");
  if (h.NGeo < 1) throw std::runtime_error("Ngeo must be >= 1");
  const long long ng3 = (h.NGeo + 1) * (h.NGeo + 1) * (h.NGeo + 1);
  const long long nSides = (long long)ds[0], nNodes = (long long)dn[0];
  for (long long e = 0; e < h.nElems; ++e) {
    const long long* ei = &h.elemInfo[(size_t)e * 6];
    if (!is_hexa(ei[0])) throw std::runtime_error("element " + std::to_string(e + 1) + " is not a hexahedron (type " + std::to_string(ei[0]) + ")");
    if (ei[3] - ei[2] < 6 || ei[2] < 0 || ei[3] > nSides) throw std::runtime_error("ElemInfo side range out of bounds");
    if (ei[5] - ei[4] != ng3 || ei[4] < 0 || ei[5] > nNodes) throw std::runtime_error("ElemInfo node range does not match Ngeo");
  }
  for (long long s = 0; s < nSides; ++s) {
    const long long* si = &h.sideInfo[(size_t)s * 5];
    if (si[2] < -3 || si[2] > h.nElems) throw std::runtime_error("SideInfo neighbour element out of range");
    if (si[4] < 0 || si[4] > h.nBCs) throw std::runtime_error("SideInfo BC index out of range");
  }
  return h;
}

}  // namespace

extern "C" {

const char* fg_io_last_error(void) { return g_ioerr.c_str(); }

int fg_hopr_sizes(const char* path, int* out) {
  if (!path || !out) return io_fail(FG_ERR_CONFIG, "fg_hopr_sizes: null argument");
  try {
    const Hopr h = read_hopr(path);
    out[0] = (int)h.nElems;
    out[1] = (int)h.NGeo;
    out[2] = (int)h.nBCs;
    int nm = 0;
    for (size_t r = 0; r < h.sideInfo.size() / 5; ++r) nm += h.sideInfo[r * 5 + 2] < 0;
    out[3] = nm;
  } catch (std::exception& e) {
    return io_fail(FG_ERR_MESH, e.what());
  }
  return FG_OK;
}

int fg_hopr_read(const char* path, double* NodeCoords, int* ElemNb, int* BoundaryType, char* BCNames, int* Mortars) {
  if (!path || !NodeCoords || !ElemNb) return io_fail(FG_ERR_CONFIG, "fg_hopr_read: null argument");
  try {
    const Hopr h = read_hopr(path);
    const long long ng3 = (h.NGeo + 1) * (h.NGeo + 1) * (h.NGeo + 1);
    // NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems): the element's nodes in file order (mesh_readin.f90:473-474)
    for (long long e = 0; e < h.nElems; ++e) {
      const long long first = h.elemInfo[(size_t)e * 6 + 4];
      for (long long k = 0; k < ng3 * 3; ++k) NodeCoords[(size_t)e * ng3 * 3 + k] = h.nodes[(size_t)first * 3 + k];
    }
    // BC types: BoundaryType(BC_TYPE, BC_STATE) = BCType(1), BCType(3) (mesh_readin.f90:171-172)
    for (long long b = 0; b < h.nBCs; ++b) {
      if (BoundaryType) {
        BoundaryType[b * 2 + 0] = (int)h.bcType[(size_t)b * 4 + 0];
        BoundaryType[b * 2 + 1] = (int)h.bcType[(size_t)b * 4 + 2];
      }
      if (BCNames) {
        std::memset(BCNames + b * 256, 0, 256);
        std::memcpy(BCNames + b * 256, h.bcNames[b].data(), std::min<size_t>(h.bcNames[b].size(), 255));
      }
    }
    // connections (mesh_readin.f90:310-456): an inner side, or a BC side of type 0, 1 (periodic) or 100, is
    // connected to its neighbour element's side 10*nbLocSide+flip / 10; other BC sides become boundaries.
    // A side with neighbour -type is a big mortar side, followed by its 2 or 4 small virtual sides
    int nMortar = 0;
    std::vector<std::pair<long long, int>> smallSides;  // (element, local side) of the small elements
    // element side of each slave side id (a small element's side of a mortar is found by its side id)
    std::map<long long, std::pair<long long, int>> slaveOf;
    for (long long e = 0; e < h.nElems; ++e) {
      long long row = h.elemInfo[(size_t)e * 6 + 2];
      for (int ls = 1; ls <= 6; ++ls, ++row) {
        const long long* si = &h.sideInfo[(size_t)row * 5];
        if (si[1] < 0) slaveOf[-si[1]] = {e, ls};
        if (si[2] < 0) row += si[2] == -1 ? 4 : 2;
      }
    }
    for (long long e = 0; e < h.nElems; ++e) {
      long long row = h.elemInfo[(size_t)e * 6 + 2];
      const long long last = h.elemInfo[(size_t)e * 6 + 3];
      for (int ls = 1; ls <= 6; ++ls, ++row) {
        if (row >= last) throw std::runtime_error("element " + std::to_string(e + 1) + ": fewer than six sides");
        const long long* si = &h.sideInfo[(size_t)row * 5];
        int* nb = &ElemNb[((size_t)e * 6 + ls - 1) * 3];
        if (si[2] < 0) {
          const int type = (int)-si[2], nm = type == 1 ? 4 : 2;
          if (row + nm >= last) throw std::runtime_error("mortar side without its small sides");
          if (Mortars) {
            int* mo = &Mortars[(size_t)nMortar * 15];
            for (int k = 0; k < 15; ++k) mo[k] = 0;
            mo[0] = (int)(e + 1); mo[1] = ls; mo[2] = type;
            for (int im = 0; im < nm; ++im) {
              const long long* sm = &h.sideInfo[(size_t)(row + 1 + im) * 5];
              auto it = slaveOf.find(sm[1] < 0 ? -sm[1] : sm[1]);
              if (sm[2] <= 0 || it == slaveOf.end() || it->second.first != sm[2] - 1)
                throw std::runtime_error("mortar small side without its small element side");
              mo[3 + 3 * im] = (int)sm[2];
              mo[4 + 3 * im] = it->second.second;
              smallSides.push_back(it->second);
            }
          }
          ++nMortar;
          row += nm;
          nb[0] = -1; nb[1] = 0; nb[2] = 0;
          continue;
        }
        if (si[0] < 0) {  // a small element's side of a mortar (negative side type, mesh_readin.f90:354)
          nb[0] = -1; nb[1] = 0; nb[2] = 0;
          continue;
        }
        const long long bc = si[4];
        bool connected = si[2] != 0;
        if (bc > 0) {
          const long long bt = h.bcType[(size_t)(bc - 1) * 4];
          if (bt != 0 && bt != 1 && bt != 100) connected = false;
        }
        nb[0] = connected ? (int)si[2] : 0;
        nb[1] = connected ? (int)(si[3] / 10) : 0;
        nb[2] = connected ? 0 : (int)bc;
        if (connected && (nb[1] < 1 || nb[1] > 6)) throw std::runtime_error("SideInfo neighbour side out of range");
        if (!connected && bc == 0) throw std::runtime_error("side without neighbour and without BC");
      }
    }
    for (const auto& sm : smallSides) {
      if (sm.first < 0 || sm.first >= h.nElems) throw std::runtime_error("mortar small element out of range");
      int* nb = &ElemNb[((size_t)sm.first * 6 + sm.second - 1) * 3];
      nb[0] = -1; nb[1] = 0; nb[2] = 0;
    }
  } catch (std::exception& e) {
    return io_fail(FG_ERR_MESH, e.what());
  }
  return FG_OK;
}

int fg_write_state(fg_handle* h, const char* path, const char* projectName, const char* meshFile, double time) {
  if (!h || !path) return io_fail(FG_ERR_CONFIG, "fg_write_state: null argument");
  int sz[5];
  if (int r = fg_get_sizes(h, sz)) return io_fail(r, "fg_write_state: no mesh");
  const int nE = sz[0], N = sz[3], n = N + 1;
  std::vector<double> U((size_t)nE * n * n * n * 5);
  if (int r = fg_get_state(h, U.data())) return io_fail(r, fg_last_error(h));
  fg_config cfg;
  if (int r = fg_get_config(h, &cfg)) return io_fail(r, fg_last_error(h));
  const int nodeType = cfg.NodeType;
  try {
    // WriteState / GenerateFileSkeleton / WriteHeader (hdf5_output.f90:60-188, 775-960)
    fgh5::Writer w;
    w.dataset_real("DG_Solution", {(uint64_t)nE, (uint64_t)n, (uint64_t)n, (uint64_t)n, 5}, U.data());
    // scalars as one-element arrays, as WriteAttribute writes them; Program, File_Type, Project_Name and
    // MeshFile at their trimmed length, the other strings at 255 characters
    w.attr_str("VarNames", {"Density", "MomentumX", "MomentumY", "MomentumZ", "EnergyStagnationDensity"});
    const std::string prj = projectName ? projectName : "", mesh = meshFile ? meshFile : "";
    w.attr_str("Program", {"FLEXI"}, false, 5);
    w.attr_str("File_Type", {"State"}, false, 5);
    w.attr_str("Project_Name", {prj}, false, prj.empty() ? 1 : (int)prj.size());
    w.attr_real("File_Version", {0.1});
    w.attr_int("N", {N});
    w.attr_int("Dimension", {3});
    w.attr_real("Time", {time});
    w.attr_str("MeshFile", {mesh}, false, mesh.empty() ? 1 : (int)mesh.size());
    w.attr_str("NextFile", {""});
    w.attr_str("NodeType", {nodeType == FG_NODE_GAUSS_LOBATTO ? "GAUSS-LOBATTO" : "GAUSS"});
    w.attr_int("NComputation", {N});
    const std::time_t now = std::time(nullptr);
    std::tm tm{};
    gmtime_r(&now, &tm);
    w.attr_int("TIME", {tm.tm_year + 1900, tm.tm_mon + 1, tm.tm_mday, 0, tm.tm_hour, tm.tm_min, tm.tm_sec, 0});
    w.write(path);
  } catch (std::exception& e) {
    return io_fail(FG_ERR_CONFIG, e.what());
  }
  return FG_OK;
}

int fg_read_state(fg_handle* h, const char* path, double* time) {
  if (!h || !path) return io_fail(FG_ERR_CONFIG, "fg_read_state: null argument");
  int sz[5];
  if (int r = fg_get_sizes(h, sz)) return io_fail(r, "fg_read_state: no mesh");
  const int nE = sz[0], N = sz[3], n = N + 1;
  fg_config cfg;
  if (int r = fg_get_config(h, &cfg)) return io_fail(r, fg_last_error(h));
  const int nodeType = cfg.NodeType;
  std::vector<double> U;
  try {
    // restart.f90: DG_Solution of the same N, node type and element count
    fgh5::Reader r(path);
    long long fN = -1;
    if (r.attr_int("N", fN) && fN != N)
      throw std::runtime_error("state has N = " + std::to_string(fN) + ", the solver N = " + std::to_string(N));
    std::vector<std::string> nt;
    if (r.attr_str("NodeType", nt) && !nt.empty()) {
      const std::string want = nodeType == FG_NODE_GAUSS_LOBATTO ? "GAUSS-LOBATTO" : "GAUSS";
      if (nt[0] != want) throw std::runtime_error("state has node type " + nt[0] + ", the solver " + want);
    }
    std::vector<uint64_t> d;
    U = r.read_real("DG_Solution", &d);
    if (d.size() != 5 || d[0] != (uint64_t)nE || d[1] != (uint64_t)n || d[2] != (uint64_t)n || d[3] != (uint64_t)n || d[4] != 5)
      throw std::runtime_error("DG_Solution does not match the mesh (nElems, N)");
    double t = 0.;
    if (time) *time = r.attr_real("Time", t) ? t : 0.;
  } catch (std::exception& e) {
    return io_fail(FG_ERR_MESH, e.what());
  }
  if (int rc = fg_set_state(h, U.data())) return io_fail(rc, fg_last_error(h));
  return FG_OK;
}

}  // extern "C"
