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
