"""Synthetic hexahedral box meshes in the form FLEXI reads from a HOPR mesh file.

FLEXI's meshes come from the external HOPR generator as HDF5 files (src/mesh/mesh_readin.f90:197:
NodeCoords on equidistant NGeo points per element, element/side connectivity, BC names and types).
This module produces the same information in memory for Cartesian boxes, optionally curved or
stretched by a coordinate map:

* ``node_coords``   (nElems, NGeo+1, NGeo+1, NGeo+1, 3) -- Fortran NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems)
* ``elem_nb``       (nElems, 6, 3) int32 -- per FLEXI local side (flexi.h:90-95): neighbour element
  (1-based, 0 for a boundary side), neighbour local side, BC index (1-based, 0 for inner sides)
* ``boundary_type`` (nBCs, 2) int32 -- BoundaryType(BC_TYPE, BC_STATE)
* ``ref_state_prim`` (nRefStates, 6) -- RefStatePrim(rho, v1, v2, v3, p, T)

Periodic directions are connected element-to-element (FLEXI treats periodic sides as inner sides,
prepare_mesh.f90:98-142). Elements are numbered lexicographically (x fastest).
"""
from dataclasses import dataclass, field

import numpy as np

# FLEXI local side ids (src/flexi.h:90-95)
ZETA_MINUS, ETA_MINUS, XI_PLUS, ETA_PLUS, XI_MINUS, ZETA_PLUS = 1, 2, 3, 4, 5, 6


@dataclass
class BoxMesh:
    n_elems: int
    ngeo: int
    node_coords: np.ndarray
    elem_nb: np.ndarray
    boundary_type: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    ref_state_prim: np.ndarray = field(default_factory=lambda: np.zeros((0, 6)))
    elem_inst: np.ndarray = None
    description: str = ""
    bc_names: list = None
    # mortar interfaces (nMortars, 15) int32: big element (1-based), its local side, type (1: 1->4, 2: 1->2 in
    # eta, 3: 1->2 in xi), then per small side: small element (1-based), its local side, 0; the elem_nb
    # entries of these sides are -1
    mortars: np.ndarray = None


def cartesian_box(nelems, lower, upper, ngeo=1, periodic=(True, True, True), mapping=None, wall_bc=None, ref_state_prim=None):
    """Box [lower, upper] with nelems=(nx,ny,nz) hexahedra of polynomial mapping degree ngeo.

    mapping: optional callable (x, y, z) -> (X, Y, Z) on arrays, applied to the equidistant node
    positions of the straight-sided element (curved or stretched meshes).
    wall_bc: (type, state) used on all non-periodic boundaries (e.g. (4, 1) isothermal wall).
    """
    nx, ny, nz = (int(v) for v in nelems)
    ng = ngeo + 1
    lo = np.asarray(lower, float)
    hi = np.asarray(upper, float)
    h = (hi - lo) / np.array([nx, ny, nz], float)
    xi = np.arange(ng) / ngeo
    ne = nx * ny * nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ix, iy, iz = (a.transpose(2, 1, 0).reshape(-1) for a in (ix, iy, iz))  # element id = ix + nx*(iy + ny*iz)
    # node (i,j,k) of element e at index [e, k, j, i]
    X = lo[0] + (ix[:, None, None, None] + xi[None, None, None, :]) * h[0]
    Y = lo[1] + (iy[:, None, None, None] + xi[None, None, :, None]) * h[1]
    Z = lo[2] + (iz[:, None, None, None] + xi[None, :, None, None]) * h[2]
    X, Y, Z = np.broadcast_arrays(X, Y, Z)
    if mapping is not None:
        X, Y, Z = mapping(X, Y, Z)
    node_coords = np.stack([X, Y, Z], axis=-1).astype(np.float64)
    nb = np.zeros((ne, 6, 3), np.int32)
    btypes = []
    if wall_bc is not None:
        btypes.append(tuple(wall_bc))
    dims = (nx, ny, nz)
    idx = (ix, iy, iz)

    def eid(a, b, c):
        return a + nx * (b + ny * c)

    pairs = [(0, XI_MINUS, XI_PLUS), (1, ETA_MINUS, ETA_PLUS), (2, ZETA_MINUS, ZETA_PLUS)]
    for d, sm, sp in pairs:
        for side, step, other in ((sm, -1, sp), (sp, +1, sm)):
            coord = [idx[0].copy(), idx[1].copy(), idx[2].copy()]
            coord[d] = coord[d] + step
            inside = (coord[d] >= 0) & (coord[d] < dims[d])
            if periodic[d]:
                coord[d] %= dims[d]
                inside[:] = True
            nbe = eid(*coord) + 1
            nb[:, side - 1, 0] = np.where(inside, nbe, 0)
            nb[:, side - 1, 1] = np.where(inside, other, 0)
            if not inside.all():
                if wall_bc is None:
                    raise ValueError("non-periodic direction needs wall_bc")
                nb[:, side - 1, 2] = np.where(inside, 0, 1)
    bt = np.array(btypes, np.int32).reshape(-1, 2)
    rs = np.zeros((0, 6)) if ref_state_prim is None else np.asarray(ref_state_prim, float).reshape(-1, 6)
    return BoxMesh(ne, ngeo, node_coords, nb, bt, rs)


def tgv_box(n_per_dir, ngeo=1, perturb=0.0, seed=0):
    """Periodic [-pi, pi]^3 Taylor-Green box. perturb > 0 curves the mesh with
    x_i += perturb * (2 pi / n) * prod_j sin(x_j + phi_ij), phases phi seeded; periodic by construction."""
    n = int(n_per_dir)
    mapping = None
    if perturb:
        rng = np.random.default_rng(seed)
        phi = rng.uniform(0.0, 2.0 * np.pi, size=(3, 3))
        amp = perturb * (2.0 * np.pi / n)

        def mapping(x, y, z):
            out = []
            for i, base in enumerate((x, y, z)):
                s = np.sin(x + phi[i, 0]) * np.sin(y + phi[i, 1]) * np.sin(z + phi[i, 2])
                out.append(base + amp * s)
            return tuple(out)
    m = cartesian_box((n, n, n), (-np.pi,) * 3, (np.pi,) * 3, ngeo=ngeo, mapping=mapping)
    m.description = f"periodic TGV box {n}^3, NGeo={ngeo}, perturbation={perturb}, seed={seed}"
    return m


def mortar_box(n_per_dir, perturb=0.0, seed=0):
    """Periodic [-pi, pi]^3 box of n^3 cells (n even) with mortar interfaces: the z-layers of cells alternate
    between one element per cell (even layers) and four elements of half the width in x and y (odd
    layers), so that both zeta faces of every coarse element are big mortar sides of type 1 (1->4) and the
    fine elements meet conformingly among themselves. 2.5 n^3 elements, n^3 mortars, NGeo=1.
    perturb > 0 displaces x and y by perturb * (2 pi / n) * prod_j sin(x_j + phi_ij) (phases seeded, periodic),
    evaluated at the coarse grid's corners and interpolated bilinearly in x and y to the fine nodes, so that
    the small faces still tile their big faces exactly."""
    n = int(n_per_dir)
    if n < 2 or n % 2:
        raise ValueError("mortar_box needs an even number of cells per direction")
    h = 2.0 * np.pi / n
    coarse, fine = {}, {}
    boxes = []  # (x0, y0, z0, hx, hy) per element, z-height h
    for k in range(n):
        for j in range(n):
            for i in range(n):
                if k % 2 == 0:
                    coarse[(i, j, k)] = len(boxes)
                    boxes.append((-np.pi + i * h, -np.pi + j * h, -np.pi + k * h, h, h))
                else:
                    for b in range(2):
                        for a in range(2):
                            fine[(2 * i + a, 2 * j + b, k)] = len(boxes)
                            boxes.append((-np.pi + (2 * i + a) * h / 2, -np.pi + (2 * j + b) * h / 2, -np.pi + k * h, h / 2, h / 2))
    ne = len(boxes)
    B = np.array(boxes)
    xi = np.array([0.0, 1.0])
    X = B[:, 0, None, None, None] + xi[None, None, None, :] * B[:, 3, None, None, None]
    Y = B[:, 1, None, None, None] + xi[None, None, :, None] * B[:, 4, None, None, None]
    Z = B[:, 2, None, None, None] + xi[None, :, None, None] * h
    X, Y, Z = np.broadcast_arrays(X, Y, Z)
    X, Y = X.copy(), Y.copy()
    if perturb:
        rng = np.random.default_rng(seed)
        phi = rng.uniform(0.0, 2.0 * np.pi, size=(2, 3))
        amp = perturb * h

        def disp(x, y, z, c):
            return amp * np.sin(x + phi[c, 0]) * np.sin(y + phi[c, 1]) * np.sin(z + phi[c, 2])
        # displacement of the coarse grid's corner nodes, interpolated bilinearly in x and y at the fine nodes
        gx = (X + np.pi) / h
        gy = (Y + np.pi) / h
        x0, y0 = np.floor(gx + 1e-9), np.floor(gy + 1e-9)
        fx, fy = gx - x0, gy - y0
        for c, A in ((0, X), (1, Y)):
            d = 0.0
            for dx, wx in ((0, 1 - fx), (1, fx)):
                for dy, wy in ((0, 1 - fy), (1, fy)):
                    d = d + wx * wy * disp(-np.pi + (x0 + dx) * h, -np.pi + (y0 + dy) * h, Z, c)
            A += d
    node_coords = np.stack([X, Y, Z], axis=-1).astype(np.float64)
    nb = np.zeros((ne, 6, 3), np.int32)
    mortars = []
    for (i, j, k), e in coarse.items():
        nb[e, XI_MINUS - 1] = (coarse[((i - 1) % n, j, k)] + 1, XI_PLUS, 0)
        nb[e, XI_PLUS - 1] = (coarse[((i + 1) % n, j, k)] + 1, XI_MINUS, 0)
        nb[e, ETA_MINUS - 1] = (coarse[(i, (j - 1) % n, k)] + 1, ETA_PLUS, 0)
        nb[e, ETA_PLUS - 1] = (coarse[(i, (j + 1) % n, k)] + 1, ETA_MINUS, 0)
        nb[e, ZETA_MINUS - 1] = (-1, 0, 0)
        nb[e, ZETA_PLUS - 1] = (-1, 0, 0)
        # zeta+ side: p ~ x, q ~ y (small side im = a + 2b); zeta- side: p ~ y, q ~ x (im = b + 2a)
        up = [0] * 4
        dn = [0] * 4
        for b in range(2):
            for a in range(2):
                up[a + 2 * b] = fine[(2 * i + a, 2 * j + b, (k + 1) % n)]
                dn[b + 2 * a] = fine[(2 * i + a, 2 * j + b, (k - 1) % n)]
        mortars.append([e + 1, ZETA_PLUS, 1] + sum(([s + 1, ZETA_MINUS, 0] for s in up), []))
        mortars.append([e + 1, ZETA_MINUS, 1] + sum(([s + 1, ZETA_PLUS, 0] for s in dn), []))
    m2 = 2 * n
    for (I, J, k), e in fine.items():
        nb[e, XI_MINUS - 1] = (fine[((I - 1) % m2, J, k)] + 1, XI_PLUS, 0)
        nb[e, XI_PLUS - 1] = (fine[((I + 1) % m2, J, k)] + 1, XI_MINUS, 0)
        nb[e, ETA_MINUS - 1] = (fine[(I, (J - 1) % m2, k)] + 1, ETA_PLUS, 0)
        nb[e, ETA_PLUS - 1] = (fine[(I, (J + 1) % m2, k)] + 1, ETA_MINUS, 0)
        nb[e, ZETA_MINUS - 1] = (-1, 0, 0)
        nb[e, ZETA_PLUS - 1] = (-1, 0, 0)
    m = BoxMesh(ne, 1, node_coords, nb, np.zeros((0, 2), np.int32), np.zeros((0, 6)),
                description=f"periodic mortar box {n}^3 cells ({ne} elements, {len(mortars)} mortars), perturbation={perturb}",
                mortars=np.array(mortars, np.int32))
    return m


def channel_box(nelems=(24, 12, 12), beta=1.5, ngeo=None, t_wall=1.0, rho_wall=1.0, p_wall=1.0):
    """Channel [0,2pi]x[-1,1]x[0,pi] with isothermal no-slip walls (BC type 4) at y=+-1, periodic in x and z,
    y-stretched by y = tanh(beta*eta)/tanh(beta) (elements cluster at the walls)."""
    if ngeo is None:
        ngeo = 2

    def mapping(x, y, z):
        return x, np.tanh(beta * y) / np.tanh(beta), z

    refstate = np.array([[rho_wall, 0.0, 0.0, 0.0, p_wall, t_wall]])
    m = cartesian_box(nelems, (0.0, -1.0, 0.0), (2.0 * np.pi, 1.0, np.pi), ngeo=ngeo, periodic=(True, False, True),
                      mapping=mapping, wall_bc=(4, 1), ref_state_prim=refstate)
    m.description = f"channel {nelems}, tanh stretching beta={beta}, NGeo={ngeo}, isothermal walls T={t_wall}"
    return m


def concatenate(meshes):
    """Ensemble mesh: independent instances side by side (elements of instance i are contiguous)."""
    ngeo = meshes[0].ngeo
    if any(m.ngeo != ngeo for m in meshes):
        raise ValueError("all instances need the same NGeo")
    coords, nbs, inst, mortars = [], [], [], []
    off = 0
    for i, m in enumerate(meshes):
        if len(m.boundary_type):
            raise ValueError("ensembles of periodic instances only")
        coords.append(m.node_coords)
        nb = m.elem_nb.copy()
        nb[:, :, 0] = np.where(nb[:, :, 0] > 0, nb[:, :, 0] + off, nb[:, :, 0])  # 0 boundary, -1 mortar side
        nbs.append(nb)
        if m.mortars is not None and len(m.mortars):
            mo = np.array(m.mortars, np.int32).copy()
            for c in (0, 3, 6, 9, 12):  # element ids of the big side and the small sides
                mo[:, c] = np.where(mo[:, c] > 0, mo[:, c] + off, mo[:, c])
            mortars.append(mo)
        inst.append(np.full(m.n_elems, i, np.int32))
        off += m.n_elems
    out = BoxMesh(off, ngeo, np.concatenate(coords), np.concatenate(nbs), mortars=np.concatenate(mortars) if mortars else None)
    out.elem_inst = np.concatenate(inst)
    out.description = f"ensemble of {len(meshes)} instances, {off} elements"
    return out


def read_hopr(path, ref_state_prim=None, boundary=None):
    """A HOPR mesh file (HDF5) as FLEXI's ReadMesh/ReadBCs read it (mesh_readin.f90:125-500), through the
    library's own reader (fg_hopr_sizes / fg_hopr_read): hexahedra, conforming and mortar interfaces.

    boundary: optional {BC name: (BC_TYPE, BC_STATE)} overrides, as the BoundaryName / BoundaryType
    keys of the parameter file replace the types stored in the mesh (mesh_readin.f90:150-172).
    ref_state_prim: RefStatePrim(rho, v1, v2, v3, p, T) rows the BC states refer to."""
    import ctypes

    from . import _lib
    L = _lib.load()
    b = str(path).encode()
    sizes = np.zeros(4, np.int32)
    if L.fg_hopr_sizes(b, sizes.ctypes.data) != 0:
        raise ValueError(L.fg_io_last_error().decode())
    ne, ng, nbc, nmo = (int(v) for v in sizes)
    mortars = np.zeros((max(nmo, 1), 15), np.int32)
    nc = np.zeros((ne, ng + 1, ng + 1, ng + 1, 3))
    nb = np.zeros((ne, 6, 3), np.int32)
    bt = np.zeros((max(nbc, 1), 2), np.int32)
    names = ctypes.create_string_buffer(256 * max(nbc, 1))
    if L.fg_hopr_read(b, nc.ctypes.data, nb.ctypes.data, bt.ctypes.data, names, mortars.ctypes.data) != 0:
        raise ValueError(L.fg_io_last_error().decode())
    mortars = mortars[:nmo]
    bc_names = [names.raw[i * 256:(i + 1) * 256].split(b"\0")[0].decode() for i in range(nbc)]
    bt = bt[:nbc]
    for name, (t, st) in (boundary or {}).items():
        matches = [i for i, nm in enumerate(bc_names) if nm.lower() == name.lower()]
        if not matches:
            raise KeyError(f"no boundary {name!r} in {path} (boundaries: {bc_names})")
        bt[matches[0]] = (t, st)
    rs = np.zeros((0, 6)) if ref_state_prim is None else np.asarray(ref_state_prim, np.float64).reshape(-1, 6)
    return BoxMesh(ne, ng, nc, nb, bt, rs, description=f"HOPR mesh {path}", bc_names=bc_names, mortars=mortars if nmo else None)
