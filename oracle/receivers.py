"""Receivers, restated in float64 (TEST INFRASTRUCTURE ONLY).

Follows src/Kernels/Receiver.cpp:118-214 (per step: CK derivatives of the receiver's cell at the
step start, Taylor expansion at each sampling time inside the step, projection onto the basis
functions at the point; rotation and strain from the basis gradients, :271-302) and
src/Numerical/Transformation.cpp:47-64 (reference coordinates of the point).
"""
import math

import numpy as np

from . import dg_setup


def locate(coords, points, tol=1e-10):
    """Lowest id of the cells (coords [n, 4, 3]) containing each point, and its reference coordinates."""
    v0 = coords[:, 0]
    J = np.stack([coords[:, 1] - v0, coords[:, 2] - v0, coords[:, 3] - v0], axis=2)  # [n, 3(x), 3(k)]
    Ji = np.linalg.inv(J)
    cells, xez = [], []
    for p in np.asarray(points, float):
        s = np.einsum("nkx,nx->nk", Ji, p - v0)
        ok = (s >= -tol).all(axis=1) & (s.sum(axis=1) <= 1 + tol)
        idx = np.nonzero(ok)[0]
        c = int(idx[0]) if len(idx) else -1
        cells.append(c)
        xez.append(s[c] if c >= 0 else np.zeros(3))
    return np.array(cells), np.array(xez)


def basis_at(order, xez, cell_coords):
    """phi [B] and global gradients dphi [3, B] (complex-step derivatives of the Dubiner basis)."""
    idx = dg_setup.basis_indices3(order)
    h = 1e-30
    phi = np.array([float(np.real(dg_setup.tet_dubiner(i, j, k, *(np.array([x], complex) for x in xez)))[0])
                    for (i, j, k) in idx])
    dref = np.zeros((3, len(idx)))
    for r in range(3):
        z = [np.array([x], complex) for x in xez]
        z[r] = z[r] + 1j * h
        dref[r] = [float(np.imag(dg_setup.tet_dubiner(i, j, k, *z))[0]) / h for (i, j, k) in idx]
    v = cell_coords
    J = np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]], axis=1)
    grad = np.linalg.inv(J)  # grad[r, x] = d xi_r / d x
    return phi, grad.T @ dref


def sample(order, derivs, phi, dphi, offsets, qmask=0x1FF, rotation=False, strain=False, visco=False):
    """Rows (time offset, kept quantities, rot1-3, strain 6) of one receiver for each offset.
    visco: derivatives of the viscoelastic update, [order][27][B] (the nine elastic quantities
    first, every stage with all basis rows)."""
    blocks, off = [], 0
    for i in range(order):
        b = len(phi) if visco else dg_setup.nbasis3(order - i)
        nq = 27 if visco else 9
        blocks.append(np.asarray(derivs[off: off + nq * b], float).reshape(nq, b)[:9])
        off += nq * b
    rows = []
    for t in offsets:
        B = len(phi)
        q = np.zeros((9, B))
        for i, blk in enumerate(blocks):
            q[:, : blk.shape[1]] += t ** i / math.factorial(i) * blk
        val = q @ phi
        g = q[6:9] @ dphi.T  # g[a, x] = d v_a / d x
        row = [t] + [val[k] for k in range(9) if qmask >> k & 1]
        if rotation:
            row += [g[2, 1] - g[1, 2], g[0, 2] - g[2, 0], g[1, 0] - g[0, 1]]
        if strain:
            row += [g[0, 0], 0.5 * (g[0, 1] + g[1, 0]), 0.5 * (g[0, 2] + g[2, 0]), g[1, 1],
                    0.5 * (g[1, 2] + g[2, 1]), g[2, 2]]
        rows.append(row)
    return np.array(rows)
