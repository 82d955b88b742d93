"""Periodic cube mesh for oracle checks (TEST INFRASTRUCTURE ONLY).

Each cube of an (nx, ny, nz) grid is split into 5 tetrahedra, mirrored on cubes of odd
parity so that face diagonals match across cubes; the domain is periodic in all three
directions, so every face is an interior face.  Tetrahedra are positively oriented
(det[v1-v0, v2-v0, v3-v0] > 0), which makes the FACE2NODES normals outward.
Cells are ordered by type (parity, tet index) and then by cube, so that cells of equal
face relations are contiguous.
"""
import numpy as np

_EVEN = [
    [(0, 0, 0), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
    [(1, 0, 0), (0, 0, 0), (1, 1, 0), (1, 0, 1)],
    [(0, 1, 0), (0, 0, 0), (1, 1, 0), (0, 1, 1)],
    [(0, 0, 1), (0, 0, 0), (1, 0, 1), (0, 1, 1)],
    [(1, 1, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
]


def _tets(parity):
    out = []
    for t in _EVEN:
        pts = [((1 - a) if parity else a, b, c) for (a, b, c) in t]
        v = np.array(pts, dtype=float)
        if np.linalg.det(np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]])) < 0:
            pts[2], pts[3] = pts[3], pts[2]
        out.append(pts)
    return out


def periodic_cube(nx, ny, nz, h=100.0):
    """Returns (topology [n,4] int64 vertex ids, coords [n,4,3] float64 unwrapped)."""
    # even counts keep the alternating split conforming; >= 4 keeps periodic faces distinct
    assert min(nx, ny, nz) >= 4 and nx % 2 == 0 and ny % 2 == 0 and nz % 2 == 0
    cubes = [(i, j, k) for k in range(nz) for j in range(ny) for i in range(nx)]
    topo, coords = [], []
    for parity in (0, 1):
        for t in _tets(parity):
            for (i, j, k) in cubes:
                if (i + j + k) % 2 != parity:
                    continue
                ids, xyz = [], []
                for (a, b, c) in t:
                    gi, gj, gk = i + a, j + b, k + c
                    ids.append((gi % nx) + nx * ((gj % ny) + ny * (gk % nz)))
                    xyz.append((gi * h, gj * h, gk * h))
                topo.append(ids)
                coords.append(xyz)
    return np.array(topo, dtype=np.int64), np.array(coords, dtype=float)


def box_mesh(nx, ny, nz, h=100.0, fault_x=None, fault_y=None, fault_y_tag=65):
    """A bounded box of PUML arrays (TEST INFRASTRUCTURE ONLY): geometry [nv, 3] on the
    (nx + 1)(ny + 1)(nz + 1) grid, connect [n, 4] (the cube split above, positively oriented),
    boundary [n] (i32: 8 bits per face) with 1 (free surface) on the top z = nz h, 5 (outflow) on
    the other sides, 3 on the cube-vertex plane x = fault_x h and fault_y_tag on y = fault_y h
    (interior planes; None: none).  Cells whose tetrahedron touches both planes carry two fault faces."""
    assert nx % 2 == 0 and ny % 2 == 0 and nz % 2 == 0
    vid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    geometry = np.array([(i * h, j * h, k * h) for k in range(nz + 1) for j in range(ny + 1) for i in range(nx + 1)])
    connect, grid = [], []
    for parity in (0, 1):
        for t in _tets(parity):
            for k in range(nz):
                for j in range(ny):
                    for i in range(nx):
                        if (i + j + k) % 2 != parity:
                            continue
                        connect.append([vid(i + a, j + b, k + c) for (a, b, c) in t])
                        grid.append([(i + a, j + b, k + c) for (a, b, c) in t])
    connect = np.array(connect, dtype=np.int64)
    grid = np.array(grid)
    face2nodes = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))
    boundary = np.zeros(len(connect), dtype=np.uint32)
    for c in range(len(connect)):
        for f, nodes in enumerate(face2nodes):
            g = grid[c, list(nodes)]
            code = 0
            for axis, top in ((0, nx), (1, ny), (2, nz)):
                if (g[:, axis] == 0).all() or (g[:, axis] == top).all():
                    code = 1 if axis == 2 and (g[:, 2] == nz).all() else 5
            if fault_x is not None and (g[:, 0] == fault_x).all():
                code = 3
            if fault_y is not None and (g[:, 1] == fault_y).all():
                code = fault_y_tag
            boundary[c] |= np.uint32(code) << np.uint32(8 * f)
    return geometry, connect, boundary
