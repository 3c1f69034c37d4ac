"""Synthetic tetrahedral meshes for the steady Euler path, and a Gmsh 2.2 ASCII writer.

Two families of hexahedral grids are generated and every hex is split into six
positively oriented tetrahedra (Kuhn / Freudenthal split along the (0,0,0)->(1,1,1)
diagonal, so neighbouring hexes share conforming triangular faces):

* ``bump_channel``: x in [-2, 4], y in [0, 1], z in [0, 1]; the bottom wall carries the
  bump y_b = h*cos^2(pi*(x-0.5)) for |x-0.5| < 0.5 and nodes are mapped as
  y = y_b + eta*(1 - y_b) with eta uniform.  Bottom and the two z-sides are slip walls;
  inflow, outflow and top are freestream.
* ``gaussian_box``: x, z in [-10, 10], y in [0, 10]; the bottom wall is
  y_w = 0.1*exp(-(x^2+z^2)/0.25) (slip wall), all other sides are freestream.  Cell sizes
  grow geometrically (ratio 1.05 by default) away from the bump in x and z and away from
  the wall in y.

The written files satisfy every constraint of the reference's Gmsh reader
(src/Mesh.cpp:95-558 of joel-ho/BES): single-space separators, exactly two tags per element
(physical, elementary), node ids contiguous from 1, boundary triangles listed before the
tetrahedra, a 3-D physical group so the reader infers nDim = 3, and the boundary names
SLIP_WALL / FREESTREAM that src/Options.cpp:22-26 maps.
"""
from __future__ import annotations

import itertools
import math
import os
from dataclasses import dataclass

import numpy as np

SLIP_WALL = 1
FREESTREAM = 2
FLUID = 3
BOUNDARY_NAMES = {SLIP_WALL: "SLIP_WALL", FREESTREAM: "FREESTREAM"}


@dataclass
class TetMesh:
    """Vertices (float64, [Nv,3]), tetrahedra (int64, [Nc,4], 0-based), boundary
    triangles (int64, [Nb,3], 0-based) and their boundary tag (1 slip wall, 2 freestream)."""

    nodes: np.ndarray
    tets: np.ndarray
    btris: np.ndarray
    btags: np.ndarray
    name: str = "mesh"

    @property
    def n_cells(self) -> int:
        return int(self.tets.shape[0])

    @property
    def n_boundary(self) -> int:
        return int(self.btris.shape[0])

    @property
    def dim(self) -> int:
        """3 for tetrahedra ([Nc,4], boundary triangles); 2 for triangles ([Nc,3], boundary
        lines [Nb,2], z = 0)."""
        return 3 if self.tets.shape[1] == 4 else 2

    @property
    def n_faces(self) -> int:
        return ((self.dim + 1) * self.n_cells + self.n_boundary) // 2


def _kuhn_tets() -> np.ndarray:
    """Six tets of the unit cube as corner indices (bit0 = i, bit1 = j, bit2 = k),
    each positively oriented (det[v1-v0, v2-v0, v3-v0] > 0)."""
    out = []
    for perm in itertools.permutations(range(3)):
        c0 = 0
        c1 = 1 << perm[0]
        c2 = c1 | (1 << perm[1])
        c3 = 7
        # parity of the permutation fixes the orientation of the path simplex
        inv = sum(1 for a in range(3) for b in range(a + 1, 3) if perm[a] > perm[b])
        if inv % 2 == 1:
            c1, c2 = c2, c1
        out.append((c0, c1, c2, c3))
    return np.array(out, dtype=np.int64)


def _structured_tets(nx: int, ny: int, nz: int) -> np.ndarray:
    """Kuhn-split tetrahedra of an nx*ny*nz hex grid, hex order x fastest, 0-based node ids
    with node(i,j,k) = i + (nx+1)*(j + (ny+1)*k)."""
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = (i * sx + j * sy + k * sz).transpose(2, 1, 0).reshape(-1)  # x fastest
    corner_off = np.array([(c & 1) * sx + ((c >> 1) & 1) * sy + ((c >> 2) & 1) * sz
                           for c in range(8)], dtype=np.int64)
    kt = _kuhn_tets()
    tets = base[:, None, None] + corner_off[kt][None, :, :]
    return tets.reshape(-1, 4)


def _boundary_tris(nx: int, ny: int, nz: int, tag_of_side) -> tuple[np.ndarray, np.ndarray]:
    """Boundary triangles of the hex grid split along each quad's lo->hi diagonal (the
    diagonal the Kuhn split induces on every cube face).  ``tag_of_side(axis, side)``
    returns the boundary tag of the side (axis 0/1/2, side 0 = min, 1 = max)."""
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    strides = (sx, sy, sz)
    dims = (nx, ny, nz)
    tris, tags = [], []
    for axis in range(3):
        u, v = [a for a in range(3) if a != axis]
        for side in range(2):
            fixed = 0 if side == 0 else dims[axis]
            iu, iv = np.meshgrid(np.arange(dims[u]), np.arange(dims[v]), indexing="ij")
            iu = iu.T.reshape(-1)
            iv = iv.T.reshape(-1)
            lo = fixed * strides[axis] + iu * strides[u] + iv * strides[v]
            hi = lo + strides[u] + strides[v]
            t1 = np.stack([lo, lo + strides[u], hi], axis=1)
            t2 = np.stack([lo, lo + strides[v], hi], axis=1)
            t = np.stack([t1, t2], axis=1).reshape(-1, 3)
            tris.append(t)
            tags.append(np.full(t.shape[0], tag_of_side(axis, side), dtype=np.int64))
    return np.concatenate(tris), np.concatenate(tags)


def bump_channel(nx: int = 60, ny: int = 20, nz: int = 10, h: float = 0.04) -> TetMesh:
    """Bump channel x in [-2,4], y in [0,1], z in [0,1] with a cos^2 bump of height h."""
    x = -2.0 + 6.0 * np.arange(nx + 1, dtype=np.float64) / nx
    eta = np.arange(ny + 1, dtype=np.float64) / ny
    z = np.arange(nz + 1, dtype=np.float64) / nz
    yb = np.where(np.abs(x - 0.5) < 0.5, h * np.cos(np.pi * (x - 0.5)) ** 2, 0.0)
    X = np.broadcast_to(x[None, None, :], (nz + 1, ny + 1, nx + 1))
    Y = yb[None, None, :] + eta[None, :, None] * (1.0 - yb[None, None, :])
    Y = np.broadcast_to(Y, (nz + 1, ny + 1, nx + 1))
    Z = np.broadcast_to(z[:, None, None], (nz + 1, ny + 1, nx + 1))
    nodes = np.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], axis=1).copy()

    def tag(axis, side):
        if axis == 1 and side == 0:
            return SLIP_WALL  # bottom wall with the bump
        if axis == 2:
            return SLIP_WALL  # z sides
        return FREESTREAM  # inflow, outflow, top

    btris, btags = _boundary_tris(nx, ny, nz, tag)
    return TetMesh(nodes, _structured_tets(nx, ny, nz), btris, btags,
                   name=f"bump_channel_{nx}x{ny}x{nz}_h{h:g}")


def bump_channel_2d(nx: int = 60, ny: int = 20, h: float = 0.04) -> TetMesh:
    """2-D bump channel: x in [-2, 4], y in [0, 1] over the bump y_b = h cos^2(pi (x - 0.5))
    for |x - 0.5| < 0.5, nodes mapped y = y_b + eta (1 - y_b); each quad split into two
    counter-clockwise triangles.  Bottom: slip wall; inflow, outflow and top: freestream."""
    x = np.linspace(-2.0, 4.0, nx + 1)
    eta = np.linspace(0.0, 1.0, ny + 1)
    yb = np.where(np.abs(x - 0.5) < 0.5, h * np.cos(np.pi * (x - 0.5)) ** 2, 0.0)
    X, E = np.meshgrid(x, eta, indexing="ij")
    Y = yb[:, None] + E * (1.0 - yb[:, None])
    nodes = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)

    def n(i, j):
        return i * (ny + 1) + j

    tris = []
    for i in range(nx):
        for j in range(ny):
            a, b, c, d = n(i, j), n(i + 1, j), n(i + 1, j + 1), n(i, j + 1)
            tris += [(a, b, c), (a, c, d)]
    lines, tags = [], []
    for i in range(nx):
        lines.append((n(i, 0), n(i + 1, 0)))
        tags.append(SLIP_WALL)
        lines.append((n(i, ny), n(i + 1, ny)))
        tags.append(FREESTREAM)
    for j in range(ny):
        lines.append((n(0, j), n(0, j + 1)))
        tags.append(FREESTREAM)
        lines.append((n(nx, j), n(nx, j + 1)))
        tags.append(FREESTREAM)
    return TetMesh(nodes, np.array(tris, np.int64), np.array(lines, np.int64),
                   np.array(tags, np.int64), name=f"bump_channel_2d_{nx}x{ny}_h{h}")


def _stretched_symmetric(n: int, half: float, ratio: float) -> np.ndarray:
    """n cells over [-half, half], smallest at 0, sizes growing by ``ratio`` outward."""
    assert n % 2 == 0, "need an even cell count for a grid symmetric about the bump"
    m = n // 2
    h0 = half * (ratio - 1.0) / (ratio ** m - 1.0) if ratio != 1.0 else half / m
    pos = np.concatenate([[0.0], np.cumsum(h0 * ratio ** np.arange(m))])
    pos[-1] = half
    return np.concatenate([-pos[::-1], pos[1:]])


def _stretched_one_sided(n: int, length: float, ratio: float) -> np.ndarray:
    h0 = length * (ratio - 1.0) / (ratio ** n - 1.0) if ratio != 1.0 else length / n
    pos = np.concatenate([[0.0], np.cumsum(h0 * ratio ** np.arange(n))])
    pos[-1] = length
    return pos


def gaussian_box(nx: int = 100, ny: int = 50, nz: int = 100, ratio: float = 1.05,
                 amp: float = 0.1, width2: float = 0.25) -> TetMesh:
    """Flat plate with a Gaussian bump, x,z in [-10,10], y in [0,10]."""
    x = _stretched_symmetric(nx, 10.0, ratio)
    z = _stretched_symmetric(nz, 10.0, ratio)
    eta = _stretched_one_sided(ny, 10.0, ratio)
    Xg, Zg = np.meshgrid(x, z, indexing="xy")  # [nz+1, nx+1]
    yw = amp * np.exp(-(Xg ** 2 + Zg ** 2) / width2)
    Y = yw[:, None, :] + (eta[None, :, None] / 10.0) * (10.0 - yw[:, None, :])
    X = np.broadcast_to(x[None, None, :], Y.shape)
    Z = np.broadcast_to(z[:, None, None], Y.shape)
    nodes = np.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], axis=1).copy()

    def tag(axis, side):
        return SLIP_WALL if (axis == 1 and side == 0) else FREESTREAM

    btris, btags = _boundary_tris(nx, ny, nz, tag)
    return TetMesh(nodes, _structured_tets(nx, ny, nz), btris, btags,
                   name=f"gaussian_box_{nx}x{ny}x{nz}_r{ratio:g}")


def tet_signed_volumes(mesh: TetMesh) -> np.ndarray:
    p = mesh.nodes[mesh.tets]
    a, b, c = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    return np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0


def _fmt_coord(v: float) -> str:
    return repr(float(v))


def write_gmsh(mesh: TetMesh, path: str) -> None:
    """Write Gmsh 2.2 ASCII: boundary faces first (triangles; lines in 2-D), then the cells
    (tets; triangles in 2-D), single spaces, two tags."""
    nv = mesh.nodes.shape[0]
    nb = mesh.btris.shape[0]
    nc = mesh.tets.shape[0]
    d = mesh.dim
    ftype, ctype = (2, 4) if d == 3 else (1, 2)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
        f.write("$PhysicalNames\n3\n")
        f.write(f'{d - 1} {SLIP_WALL} "SLIP_WALL"\n{d - 1} {FREESTREAM} "FREESTREAM"\n'
                f'{d} {FLUID} "FLUID"\n')
        f.write("$EndPhysicalNames\n")
        f.write(f"$Nodes\n{nv}\n")
        lines = []
        for i in range(nv):
            x, y, z = mesh.nodes[i]
            lines.append(f"{i + 1} {_fmt_coord(x)} {_fmt_coord(y)} {_fmt_coord(z)}\n")
            if len(lines) >= 65536:
                f.write("".join(lines))
                lines = []
        f.write("".join(lines))
        f.write("$EndNodes\n")
        f.write(f"$Elements\n{nb + nc}\n")
        eid = 1
        chunk = []
        bt = mesh.btris + 1
        for i in range(nb):
            t = bt[i]
            tag = int(mesh.btags[i])
            chunk.append(f"{eid} {ftype} 2 {tag} {tag} " + " ".join(str(v) for v in t) + "\n")
            eid += 1
            if len(chunk) >= 65536:
                f.write("".join(chunk))
                chunk = []
        tt = mesh.tets + 1
        for i in range(nc):
            t = tt[i]
            chunk.append(f"{eid} {ctype} 2 {FLUID} {FLUID} " + " ".join(str(v) for v in t) + "\n")
            eid += 1
            if len(chunk) >= 65536:
                f.write("".join(chunk))
                chunk = []
        f.write("".join(chunk))
        f.write("$EndElements\n")


def freestream_mach_vector(mach: float, pitch_deg: float = 0.0,
                           sideslip_deg: float = 0.0) -> tuple[float, float, float]:
    """Mach vector from magnitude, pitch (x-y plane) and sideslip (x-z plane)."""
    a = math.radians(pitch_deg)
    b = math.radians(sideslip_deg)
    return (mach * math.cos(a) * math.cos(b), mach * math.sin(a) * math.cos(b),
            mach * math.sin(b))


def sample_conditions(n: int, seed: int, mach=(0.3, 0.85), pitch=(-4.0, 4.0),
                      sideslip=(-4.0, 4.0)) -> np.ndarray:
    """[n,3] (Mach, pitch deg, sideslip deg) drawn uniformly from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    m = rng.uniform(mach[0], mach[1], n)
    p = rng.uniform(pitch[0], pitch[1], n)
    s = rng.uniform(sideslip[0], sideslip[1], n)
    return np.stack([m, p, s], axis=1)
