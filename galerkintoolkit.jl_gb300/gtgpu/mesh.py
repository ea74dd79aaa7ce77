"""Mesh input: Cartesian meshes with boundary faces and groups, seeded
synthetic perturbations.

``cartesian_mesh`` mirrors ``GT.cartesian_mesh(domain, cells; simplexify)``
(src/cartesian_mesh.jl:16-54): nodes are numbered x-fastest
(cartesian_chain, src/cartesian_mesh.jl:213-263), cell nodes follow the
reference cell's CartesianIndices(0:1,...) order, simplex meshes split every
cube into the 6 tetrahedra of src/domain.jl:322-342, and the boundary
barrier (src/cartesian_mesh.jl:105-181, :342-427) produces the parent
d-faces that fix the topology numbering: a local d-face of a cell is a
parent face when all its nodes touch at most 2^d cells, found cell by cell in
local-face order, and its group is "d-face-k" with k its local index.
All arrays are host numpy arrays with 1-based ids (GT convention); the
vectorised code here is independent of the CPU oracle it is tested against.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

QUAD4, HEX8, TET4 = 1, 2, 3

QUAD_EDGES = np.array([[1, 2], [3, 4], [1, 3], [2, 4]]) - 1
HEX_EDGES = np.array([[1, 2], [3, 4], [1, 3], [2, 4], [5, 6], [7, 8],
                      [5, 7], [6, 8], [1, 5], [3, 7], [2, 6], [4, 8]]) - 1
HEX_FACES = np.array([[1, 2, 3, 4], [5, 6, 7, 8], [1, 2, 5, 6],
                      [3, 4, 7, 8], [1, 3, 5, 7], [2, 4, 6, 8]]) - 1
TET_FACES = np.array([[1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]]) - 1
CUBE_TETS = np.array([[1, 2, 3, 7], [1, 2, 5, 7], [2, 3, 4, 7],
                      [2, 4, 7, 8], [2, 5, 6, 7], [2, 6, 7, 8]]) - 1


@dataclass
class Mesh:
    """A GT-style mesh: coordinates, cells and the parent boundary faces."""
    D: int
    cell_type: int
    coords: np.ndarray          # (nnodes, D) float64
    cell_nodes: np.ndarray      # (ncells, nv) int32, 1-based
    corners: np.ndarray         # parent 0-faces, 1-based node ids
    bfaces: np.ndarray          # parent (D-1)-faces, (n, nfv) 1-based
    bface_group: np.ndarray     # local face index k of group "(D-1)-face-k"
    bedges: np.ndarray          # 3-D parent 1-faces (box-edge segments)
    cells_per_dir: tuple = ()
    domain: tuple = ()
    _device: dict = field(default_factory=dict, repr=False)

    @property
    def num_nodes(self):
        return self.coords.shape[0]

    @property
    def num_cells(self):
        return self.cell_nodes.shape[0]

    def group_names(self):
        d = self.D - 1
        return ["boundary"] + [f"{d}-face-{k}" for k in sorted(set(self.bface_group.tolist()))]


def _node_grid(cells):
    D = len(cells)
    np_ = [c + 1 for c in cells]
    idx = np.indices(np_[::-1]).reshape(D, -1)[::-1]  # idx[d][node] x-fastest
    return np_, idx


def _hex_cells(cells):
    """(cell nodes 0-based, ncells x 2^D; cell coordinates, D x ncells)."""
    D = len(cells)
    np_ = [c + 1 for c in cells]
    ci = np.indices(cells[::-1]).reshape(D, -1)[::-1]  # cell coords, x-fastest
    strides = np.cumprod([1] + np_[:-1])
    nlv = 1 << D
    base = np.zeros(ci.shape[1], np.int64)
    for d in range(D):
        base += ci[d] * strides[d]
    off = np.array([sum(((lv >> d) & 1) * strides[d] for d in range(D)) for lv in range(nlv)], np.int64)
    return base[:, None] + off[None, :], ci


def _cube_face_triangles():
    """Boundary triangles of each cube face in the complexified 6-tet split:
    first-encounter order over tets and their local faces (vertex order of
    the first tet), src/topology.jl:1594-1704 applied to src/domain.jl:322-342."""
    tris = []
    keys = set()
    for t in CUBE_TETS:
        for f in TET_FACES:
            v = tuple(int(x) for x in t[f])
            k = frozenset(v)
            if k not in keys:
                keys.add(k)
                tris.append(v)
    out = []
    for face in HEX_FACES:
        fs = set(int(x) for x in face)
        out.append([tr for tr in tris if set(tr) <= fs])
    return out


def cartesian_mesh(domain, cells, simplexify=False):
    """GT.cartesian_mesh(domain, cells; simplexify) with boundary groups."""
    cells = tuple(int(c) for c in cells)
    D = len(cells)
    if D not in (2, 3):
        raise ValueError("only 2-D and 3-D meshes are supported")
    if any(c != 1 for c in cells) and any(c < 2 for c in cells):
        raise ValueError("At least 2 cells in any direction (or 1 cell in all directions)")
    if simplexify and D != 3:
        raise NotImplementedError("simplex meshes are supported in 3-D (TET4) only")
    np_, idx = _node_grid(cells)
    lo = np.array(domain[0::2], np.float64)
    hi = np.array(domain[1::2], np.float64)
    h = (hi - lo) / np.array(cells, np.float64)
    coords = np.ascontiguousarray((lo[:, None] + h[:, None] * idx).T)
    hexes, cidx = _hex_cells(cells)
    # number of hex cells around each node
    cnt = np.ones(coords.shape[0], np.int64)
    for d in range(D):
        cnt *= np.where((idx[d] == 0) | (idx[d] == cells[d]), 1, 2)
    # boundary entities lie in boundary cells only: the scans below run over
    # those (ascending, so every list keeps the order of a scan over all cells)
    onb = np.zeros(hexes.shape[0], bool)
    for d in range(D):
        onb |= (cidx[d] == 0) | (cidx[d] == cells[d] - 1)
    bcell = np.nonzero(onb)[0]
    hb = hexes[bcell]
    cc = cnt[hb]  # (boundary cells, nlv)
    # d = 0: corners, in cell order
    corners = hb[cc <= 1]
    # parent 1-faces
    ledges = QUAD_EDGES if D == 2 else HEX_EDGES
    e_ok = (cc[:, ledges[:, 0]] <= 2) & (cc[:, ledges[:, 1]] <= 2)
    ci, le = np.nonzero(e_ok)
    edges = np.stack([hb[ci, ledges[le, 0]], hb[ci, ledges[le, 1]]], 1)
    egroup = le + 1
    if D == 2:
        bfaces, bgroup, bedges = edges, egroup, np.zeros((0, 2), np.int64)
        ctype = QUAD4
        cell_nodes = hexes
    else:
        f_ok = np.all(cc[:, HEX_FACES] <= 4, axis=2)
        ci, lf = np.nonzero(f_ok)
        bedges = edges
        if not simplexify:
            bfaces = hb[ci[:, None], HEX_FACES[lf]]
            bgroup = lf + 1
            ctype = HEX8
            cell_nodes = hexes
        else:
            tri = _cube_face_triangles()
            ntri = np.array([len(t) for t in tri])
            rep = ntri[lf]
            ci2 = np.repeat(ci, rep)
            lf2 = np.repeat(lf, rep)
            sub = np.concatenate([np.arange(r) for r in rep]) if rep.size else np.zeros(0, np.int64)
            tri_arr = np.array(tri)  # (6, 2, 3)
            bfaces = hb[ci2[:, None], tri_arr[lf2, sub]]
            bgroup = lf2 + 1
            ctype = TET4
            cell_nodes = hexes[:, CUBE_TETS].reshape(-1, 4)
    i32 = lambda a: np.ascontiguousarray(np.asarray(a, np.int64) + 1, dtype=np.int32)
    return Mesh(D=D, cell_type=ctype, coords=coords, cell_nodes=i32(cell_nodes), corners=i32(corners),
                bfaces=i32(bfaces), bface_group=np.ascontiguousarray(bgroup, np.int32), bedges=i32(bedges),
                cells_per_dir=cells, domain=tuple(float(x) for x in domain))


# ---------------------------------------------------------------------------
# seeded synthetic inputs: splitmix64 keyed uniforms
# ---------------------------------------------------------------------------
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M
        z = x
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M
        return z ^ (z >> np.uint64(31))


def keyed_uniform(seed, keys):
    """u = (splitmix64(seed ^ key) >> 11) * 2^-53, elementwise over keys."""
    k = np.asarray(keys, np.uint64) ^ np.uint64(seed)
    return (_splitmix64(k) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def jitter_interior_nodes(mesh: Mesh, amplitude: float, seed: int) -> Mesh:
    """Move interior nodes by U(-a h, a h) per axis (key 4*node0+axis)."""
    cells = mesh.cells_per_dir
    D = mesh.D
    _, idx = _node_grid(cells)
    interior = np.ones(mesh.num_nodes, bool)
    for d in range(D):
        interior &= (idx[d] > 0) & (idx[d] < cells[d])
    nodes = np.nonzero(interior)[0].astype(np.uint64)
    lo = np.array(mesh.domain[0::2])
    hi = np.array(mesh.domain[1::2])
    h = (hi - lo) / np.array(cells)
    for d in range(D):
        u = keyed_uniform(seed, np.uint64(4) * nodes + np.uint64(d))
        mesh.coords[nodes.astype(np.int64), d] += amplitude * h[d] * (2.0 * u - 1.0)
    mesh._device.clear()
    return mesh


def lognormal_cells(ncells: int, sigma: float, seed: int) -> np.ndarray:
    """Per-cell exp(sigma * N(0,1)), Box-Muller of keys 2c, 2c+1 under
    seed ^ 0xC0EFF1C1E47."""
    s = int(seed) ^ 0xC0EFF1C1E47
    c = np.arange(ncells, dtype=np.uint64)
    u1 = keyed_uniform(s, np.uint64(2) * c)
    u2 = keyed_uniform(s, np.uint64(2) * c + np.uint64(1))
    z = np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(6.283185307179586 * u2)
    return np.exp(sigma * z)
