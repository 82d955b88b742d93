"""CPU oracle, set-up half: global DG matrices, mesh face relations and per-cell operators.

TEST INFRASTRUCTURE ONLY.  This module (and everything under ``oracle/``) is the
checker for the GPU path.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` may import it; the product never does.

Everything here is a float64 restatement of the reference's mathematics, derived
independently (Gauss-Legendre quadrature on collapsed coordinates) and pinned in
``tests/`` against the reference's own matrix files and unit-test golden values:

* basis ordering and Dubiner polynomials: ``src/Numerical/BasisFunction.h:133-142``,
  ``src/Numerical/Functions.cpp:63-160`` (singularity-free Jacobi recursion);
* global matrices ``kDivM, kDivMT, rDivM, rT, fMrT, fP``:
  ``codegen/matrices/matrices_{20,35,56}.xml`` as consumed by ``codegen/kernels/aderdg.py``;
  ``kDivMT`` is negated at load in ``src/Memory/GlobalData.cpp:51-61`` and returned negated here;
* face parameterisation and orientation: ``src/Numerical/Transformation.cpp:300-348``,
  ``src/Geometry/MeshTools.cpp:21-23``, ``src/Geometry/PUMLReader.cpp:151-163,414-427``;
* coefficient matrices / Godunov state / rotations:
  ``src/Equations/elastic/Model/ElasticSetup.h:27-198``, ``src/Numerical/Transformation.cpp:66-290``;
* star matrices and flux solvers: ``src/Initializer/Model/CellLocalMatrices.cpp:46-296``
  and ``codegen/kernels/aderdg.py:226-246``.

Matrix layouts follow yateto's column-major convention of the reference: a B x Nq DOF
tensor ``Q[k, p]`` has the basis index fastest.  Arrays returned here are numpy arrays
indexed ``[row, col]``.
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np
from numpy.polynomial.legendre import leggauss

FACE2NODES = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))


def nbasis3(order: int) -> int:
    return order * (order + 1) * (order + 2) // 6


def nbasis2(order: int) -> int:
    return order * (order + 1) // 2


# ---------------------------------------------------------------------------
# Dubiner basis (Functions.cpp:63-160); the recursion is evaluated on complex
# inputs so that derivatives come out exactly by the complex-step method.
# ---------------------------------------------------------------------------
def _sf_jacobi(n, a, b, x, y):
    """y^n * P_n^{(a,b)}(x / y) by the three-term recurrence (no division by y)."""
    if n == 0:
        return np.ones_like(x)
    pm1 = np.ones_like(x)
    pm = (0.5 * a - 0.5 * b) * y + (1.0 + 0.5 * (a + b)) * x
    for m in range(2, n + 1):
        pm2, pm1 = pm1, pm
        c0 = 2.0 * m + a + b
        pm = ((c0 - 1.0) * ((a * a - b * b) * y + c0 * (c0 - 2.0) * x) * pm1
              - 2.0 * (m + a - 1.0) * (m + b - 1.0) * c0 * y * y * pm2) / (2.0 * m * (m + a + b) * (c0 - 2.0))
    return pm


def tet_dubiner(i, j, k, xi, eta, zeta):
    one = np.ones_like(xi)
    return (_sf_jacobi(i, 0, 0, 2 * xi - 1 + eta + zeta, 1 - eta - zeta)
            * _sf_jacobi(j, 2 * i + 1, 0, 2 * eta - 1 + zeta, 1 - zeta)
            * _sf_jacobi(k, 2 * i + 2 * j + 2, 0, 2 * zeta - 1, one))


def tri_dubiner(i, j, xi, eta):
    return _sf_jacobi(i, 0, 0, 2 * xi - 1 + eta, 1 - eta) * _sf_jacobi(j, 2 * i + 1, 0, 2 * eta - 1, np.ones_like(eta))


def basis_indices3(order):
    """Reference ordering (BasisFunction.h:133-142): by degree, then k, then j."""
    out = []
    for o in range(order):
        for k in range(o + 1):
            for j in range(o - k + 1):
                out.append((o - j - k, j, k))
    return out


def basis_indices2(order):
    out = []
    for o in range(order):
        for j in range(o + 1):
            out.append((o - j, j))
    return out


def _quad_tet(n):
    x, w = leggauss(n)
    x = 0.5 * (x + 1.0)
    w = 0.5 * w
    a, b, c = np.meshgrid(x, x, x, indexing="ij")
    wa, wb, wc = np.meshgrid(w, w, w, indexing="ij")
    zeta = c
    eta = b * (1 - c)
    xi = a * (1 - b) * (1 - c)
    return xi.ravel(), eta.ravel(), zeta.ravel(), (wa * wb * wc * (1 - b) * (1 - c) ** 2).ravel()


def _quad_tri(n):
    x, w = leggauss(n)
    x = 0.5 * (x + 1.0)
    w = 0.5 * w
    a, b = np.meshgrid(x, x, indexing="ij")
    wa, wb = np.meshgrid(w, w, indexing="ij")
    return (a * (1 - b)).ravel(), b.ravel(), (wa * wb * (1 - b)).ravel()


def face_point(face, chi, tau):
    """Reference-tet coordinates of face-local (chi, tau) (Transformation.cpp:300-348)."""
    z = np.zeros_like(chi)
    if face == 0:
        return tau, chi, z
    if face == 1:
        return chi, z, tau
    if face == 2:
        return z, tau, chi
    return 1 - chi - tau, chi, tau


def orientation_map(h, chi, tau):
    """Neighbour-face coordinates for side orientation h (Transformation.cpp:300-322)."""
    if h == 0:
        return tau, chi
    if h == 1:
        return 1 - chi - tau, tau
    return chi, 1 - chi - tau


@lru_cache(maxsize=None)
def global_matrices(order: int) -> dict:
    """All global matrices of the reference at a given convergence order, float64.

    Returns a dict with keys kDivM, kDivMT (each a list of 3), rDivM, rT, fMrT (lists of 4),
    fP (list of 3), plus M (mass diagonal) and fM (face mass diagonal).
    kDivMT is returned with the sign the reference applies at load time.
    """
    nq = order + 4
    xi, eta, zeta, w = _quad_tet(nq)
    ids = basis_indices3(order)
    h = 1e-30
    phi = np.array([tet_dubiner(*t, xi, eta, zeta) for t in ids])
    dphi = []
    for d in range(3):
        pts = [xi.astype(complex), eta.astype(complex), zeta.astype(complex)]
        pts[d] = pts[d] + 1j * h
        dphi.append(np.array([tet_dubiner(*t, *pts).imag / h for t in ids]))
    mass = (phi * w) @ phi.T
    minv = 1.0 / np.diag(mass)
    kdivm = [minv[:, None] * ((dphi[d] * w) @ phi.T) for d in range(3)]
    kdivmt = [-(minv[:, None] * ((phi * w) @ dphi[d].T)) for d in range(3)]

    chi, tau, w2 = _quad_tri(nq)
    ids2 = basis_indices2(order)
    psi = np.array([tri_dubiner(*t, chi, tau) for t in ids2])
    fmass = np.diag((psi * w2) @ psi.T)
    rT, fMrT, rDivM = [], [], []
    for f in range(4):
        pf = np.array([tet_dubiner(*t, *face_point(f, chi, tau)) for t in ids])
        s = (psi * w2) @ pf.T
        rT.append(s / fmass[:, None])
        fMrT.append(s)
        rDivM.append(minv[:, None] * (s / fmass[:, None]).T)
    fP = []
    for hh in range(3):
        a, b = orientation_map(hh, chi, tau)
        psih = np.array([tri_dubiner(*t, a, b) for t in ids2])
        fP.append((psi * w2) @ psih.T)
    clean = lambda m: np.where(np.abs(m) < 1e-13 * max(1.0, np.abs(m).max()), 0.0, m)
    return {
        "kDivM": [clean(m) for m in kdivm],
        "kDivMT": [clean(m) for m in kdivmt],
        "rDivM": [clean(m) for m in rDivM],
        "rT": [clean(m) for m in rT],
        "fMrT": [clean(m) for m in fMrT],
        "fP": [clean(m) for m in fP],
        "M": np.diag(mass).copy(),
        "fM": fmass.copy(),
    }


def taylor_integrate(order: int, start: float, end: float) -> np.ndarray:
    """Monomial time-basis integration coefficients (TimeBasis.h:82-93): (end^{i+1}-start^{i+1})/(i+1)!."""
    return np.array([(end ** (i + 1) - start ** (i + 1)) / math.factorial(i + 1) for i in range(order)])


def taylor_point(order: int, t: float) -> np.ndarray:
    """Monomial time-basis point evaluation (TimeBasis.h:70-79): t^i / i!."""
    return np.array([t ** i / math.factorial(i) for i in range(order)])


# ---------------------------------------------------------------------------
# Mesh relations (PUMLReader.cpp:151-163, 405-427)
# ---------------------------------------------------------------------------
def face_relations(tets: np.ndarray):
    """Neighbour id, neighbour side and side orientation for every (cell, face).

    ``tets`` holds topological vertex ids [ncells, 4] (periodic identification already applied).
    Returns (neighbor[n,4] int64 (-1 on boundary), side[n,4], orient[n,4]).
    """
    n = tets.shape[0]
    key_to = {}
    for c in range(n):
        for f in range(4):
            key = tuple(sorted(int(tets[c, v]) for v in FACE2NODES[f]))
            key_to.setdefault(key, []).append((c, f))
    nb = -np.ones((n, 4), dtype=np.int64)
    side = np.zeros((n, 4), dtype=np.int64)
    orient = np.zeros((n, 4), dtype=np.int64)
    for key, lst in key_to.items():
        if len(lst) != 2:
            continue
        for (c, f), (d, j) in (tuple(lst), tuple(lst[::-1])):
            nb[c, f] = d
            side[c, f] = j
            first = int(tets[c, FACE2NODES[f][0]])
            nodes_j = [int(tets[d, v]) for v in FACE2NODES[j]]
            orient[c, f] = nodes_j.index(first)
    return nb, side, orient


# ---------------------------------------------------------------------------
# Per-cell operators (CellLocalMatrices.cpp:66-296, ElasticSetup.h)
# ---------------------------------------------------------------------------
def coefficient_matrix_T(rho, mu, lam, dim):
    """Transposed coefficient matrix A^T, B^T or C^T (ElasticSetup.h:27-77), 9x9."""
    m = np.zeros((9, 9))
    l2m = lam + 2 * mu
    ri = 1.0 / rho
    if dim == 0:
        m[6, 0], m[6, 1], m[6, 2], m[7, 3], m[8, 5] = -l2m, -lam, -lam, -mu, -mu
        m[0, 6], m[3, 7], m[5, 8] = -ri, -ri, -ri
    elif dim == 1:
        m[7, 0], m[7, 1], m[7, 2], m[6, 3], m[8, 4] = -lam, -l2m, -lam, -mu, -mu
        m[1, 7], m[3, 6], m[4, 8] = -ri, -ri, -ri
    else:
        m[8, 0], m[8, 1], m[8, 2], m[7, 4], m[6, 5] = -lam, -lam, -l2m, -mu, -mu
        m[2, 8], m[5, 6], m[4, 7] = -ri, -ri, -ri
    return m


def godunov_state(local, neighbor):
    """Transposed Godunov states (QgodLocal, QgodNeighbor) for a regular face (ElasticSetup.h:80-180).

    ``local``/``neighbor`` are (rho, mu, lambda).  Returned as numpy [i, j] = view (i, j).
    """
    rl, ml, ll = local
    rn, mn, ln = neighbor
    R = np.zeros((9, 9))
    R[0, 0] = ll + 2 * ml
    R[1, 0] = ll
    R[2, 0] = ll
    R[6, 0] = math.sqrt((ll + 2 * ml) / rl)
    R[3, 1] = ml
    R[7, 1] = math.sqrt(ml / rl)
    R[5, 2] = ml
    R[8, 2] = math.sqrt(ml / rl)
    R[4, 3] = ll + 2 * ml
    R[1, 4] = ll + 2 * ml
    R[2, 5] = ll + 2 * ml
    R[5, 6] = mn
    R[8, 6] = -math.sqrt(mn / rn)
    R[3, 7] = mn
    R[7, 7] = -math.sqrt(mn / rn)
    R[0, 8] = ln + 2 * mn
    R[1, 8] = ln
    R[2, 8] = ln
    R[6, 8] = -math.sqrt((ln + 2 * mn) / rn)
    chi = np.zeros((9, 9))
    chi[0, 0] = chi[1, 1] = chi[2, 2] = 1.0
    RT = R.T
    god = np.linalg.solve(RT, chi @ RT)
    return np.eye(9) - god, god


def free_surface_state(local):
    """Transposed Godunov state of a free-surface face (src/Model/Common.h:319-364, elastic):
    S = -(R21 R11^-1) from the traction rows (0, 3, 5) and velocity rows (6, 7, 8) of the first
    three columns of the eigenvector matrix R (ElasticSetup.h:80-118), placed as QgodLocal(t_i, v_j)
    = S(j, i), with the identity on the velocities; the neighbour state is unused (zero here)."""
    rl, ml, ll = local
    R = np.zeros((9, 3))
    R[0, 0] = ll + 2 * ml
    R[1, 0] = ll
    R[2, 0] = ll
    R[6, 0] = math.sqrt((ll + 2 * ml) / rl)
    R[3, 1] = ml
    R[7, 1] = math.sqrt(ml / rl)
    R[5, 2] = ml
    R[8, 2] = math.sqrt(ml / rl)
    tr, vel = [0, 3, 5], [6, 7, 8]
    S = -(R[vel] @ np.linalg.inv(R[tr]))
    q = np.zeros((9, 9))
    for i, t in enumerate(tr):
        for j, v in enumerate(vel):
            q[t, v] = S[j, i]
    for v in vel:
        q[v, v] = 1.0
    return q, np.zeros((9, 9))


def rotation_matrices(n, s, t):
    """Face rotation T and its inverse Tinv (ElasticSetup.h:182-198, Transformation.cpp:110-290)."""
    T = np.zeros((9, 9))
    Ti = np.zeros((9, 9))
    nx, ny, nz = n
    sx, sy, sz = s
    tx, ty, tz = t
    T[0:6, 0] = [nx * nx, ny * ny, nz * nz, ny * nx, nz * ny, nz * nx]
    T[0:6, 1] = [sx * sx, sy * sy, sz * sz, sy * sx, sz * sy, sz * sx]
    T[0:6, 2] = [tx * tx, ty * ty, tz * tz, ty * tx, tz * ty, tz * tx]
    T[0:6, 3] = [2 * nx * sx, 2 * ny * sy, 2 * nz * sz, ny * sx + nx * sy, nz * sy + ny * sz, nz * sx + nx * sz]
    T[0:6, 4] = [2 * sx * tx, 2 * sy * ty, 2 * sz * tz, sy * tx + sx * ty, sz * ty + sy * tz, sz * tx + sx * tz]
    T[0:6, 5] = [2 * nx * tx, 2 * ny * ty, 2 * nz * tz, ny * tx + nx * ty, nz * ty + ny * tz, nz * tx + nx * tz]
    for i in range(3):
        T[6 + i, 6:9] = [n[i], s[i], t[i]]
    Ti[0:6, 0] = [nx * nx, sx * sx, tx * tx, nx * sx, sx * tx, nx * tx]
    Ti[0:6, 1] = [ny * ny, sy * sy, ty * ty, ny * sy, sy * ty, ny * ty]
    Ti[0:6, 2] = [nz * nz, sz * sz, tz * tz, nz * sz, sz * tz, nz * tz]
    Ti[0:6, 3] = [2 * ny * nx, 2 * sy * sx, 2 * ty * tx, ny * sx + nx * sy, sy * tx + sx * ty, ny * tx + nx * ty]
    Ti[0:6, 4] = [2 * nz * ny, 2 * sz * sy, 2 * tz * ty, nz * sy + ny * sz, sz * ty + sy * tz, nz * ty + ny * tz]
    Ti[0:6, 5] = [2 * nz * nx, 2 * sz * sx, 2 * tz * tx, nz * sx + nx * sz, sz * tx + sx * tz, nz * tx + nx * tz]
    for i in range(3):
        Ti[6:9, 6 + i] = [n[i], s[i], t[i]]
    return T, Ti


def reference_jacobian(x, y, z):
    """Gradients of (xi, eta, zeta) w.r.t. (x, y, z) (Transformation.cpp:66-108)."""
    v = np.stack([x, y, z], axis=1)  # 4 x 3
    J = np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]], axis=1)  # columns d xyz / d ref
    Ji = np.linalg.inv(J)  # rows: grad xi, grad eta, grad zeta
    return Ji[0], Ji[1], Ji[2]


def cell_operators(coords: np.ndarray, material: np.ndarray, neighbor: np.ndarray, face_type=None, bc=None):
    """Star matrices and flux solvers for every cell.

    coords: [n, 4, 3] vertex coordinates (geometric, unwrapped); material: [n, 3] (rho, mu, lambda);
    neighbor: [n, 4] neighbour ids (material of the neighbour enters the Godunov state).
    face_type: optional [n, 4] (0 regular, 1 dynamic rupture); bc: optional [n, 4] boundary
    conditions (1: free surface, whose local flux takes free_surface_state).  Returns dict with
    star [n, 3, 9, 9], AplusT [n, 4, 9, 9], AminusT [n, 4, 9, 9] (numpy [q, p] = view (q, p)).
    """
    n = coords.shape[0]
    star = np.zeros((n, 3, 9, 9))
    ap = np.zeros((n, 4, 9, 9))
    am = np.zeros((n, 4, 9, 9))
    for c in range(n):
        rho, mu, lam = material[c]
        At = [coefficient_matrix_T(rho, mu, lam, d) for d in range(3)]
        x, y, z = coords[c, :, 0], coords[c, :, 1], coords[c, :, 2]
        grads = reference_jacobian(x, y, z)
        for e in range(3):
            star[c, e] = grads[e][0] * At[0] + grads[e][1] * At[1] + grads[e][2] * At[2]
        v = coords[c]
        ab = v[1] - v[0]
        ac = v[2] - v[0]
        ad = v[3] - v[0]
        vol = abs(np.dot(ad, np.cross(ab, ac))) / 6.0
        for f in range(4):
            a, b, cc = (v[k] for k in FACE2NODES[f])
            nrm = np.cross(b - a, cc - a)
            area = 0.5 * np.linalg.norm(nrm)
            t1 = b - a
            t2 = np.cross(nrm, t1)
            nrm = nrm / np.linalg.norm(nrm)
            t1 = t1 / np.linalg.norm(t1)
            t2 = t2 / np.linalg.norm(t2)
            nbm = material[neighbor[c, f]] if neighbor[c, f] >= 0 else material[c]
            if bc is not None and bc[c, f] == 1:
                qgl, qgn = free_surface_state(material[c])
            else:
                qgl, qgn = godunov_state(material[c], nbm)
            Atil = coefficient_matrix_T(rho, mu, lam, 0)  # isotropic: rotation has no effect
            T, Ti = rotation_matrices(nrm, t1, t2)
            scale = -2.0 * area / (6.0 * vol)
            dr = face_type is not None and face_type[c, f] == 1
            # AplusT[i,j] = fluxScale * Tinv[k,i] * (Qgod[k,q] * A~T[q,l]) * T[j,l]
            ap[c, f] = (0.0 if dr else scale) * Ti.T @ (qgl @ Atil) @ T.T
            am[c, f] = scale * Ti.T @ (qgn @ Atil) @ T.T
    return {"star": star, "AplusT": ap, "AminusT": am}


def cfl_timestep(coords: np.ndarray, vp: np.ndarray, order: int, cfl: float = 0.5) -> np.ndarray:
    """Per-cell CFL time step (GlobalTimestep.cpp:27-47)."""
    out = np.empty(coords.shape[0])
    for c in range(coords.shape[0]):
        x = coords[c]
        a = np.hstack([x, np.ones((4, 1))])
        alpha = np.linalg.det(a)
        areas = (np.linalg.norm(np.cross(x[1] - x[0], x[2] - x[0]))
                 + np.linalg.norm(np.cross(x[1] - x[0], x[3] - x[0]))
                 + np.linalg.norm(np.cross(x[2] - x[0], x[3] - x[0]))
                 + np.linalg.norm(np.cross(x[2] - x[1], x[3] - x[1])))
        insphere = abs(alpha) / areas
        out[c] = cfl * 2.0 * insphere / (vp[c] * (2 * order - 1))
    return out


# ---------------------------------------------------------------------------
# Dynamic rupture (codegen/matrices/dr_stroud_matrices_{N}.json, DynamicRuptureMatrices.cpp)
# ---------------------------------------------------------------------------
def stroud_points(order):
    """Stroud conical-product rule with order+1 points per direction on the face triangle.

    First coordinate from Gauss-Jacobi(1, 0) nodes (descending), second from Gauss-Legendre
    scaled by (1 - first); ordering and weights as codegen/matrices/dr_stroud_matrices_{N}.json.
    """
    from scipy.special import roots_jacobi, roots_legendre
    n = order + 1
    xj, wj = roots_jacobi(n, 1, 0)
    xl, wl = roots_legendre(n)
    pts, ws = [], []
    for i in reversed(range(n)):
        u = (1 + xj[i]) / 2
        for j in range(n):
            pts.append((u, (1 - u) * (1 - xl[j]) / 2))
            ws.append(wj[i] / 4 * wl[j] / 2)
    return np.array(pts), np.array(ws)


@lru_cache(maxsize=None)
def dr_matrices(order):
    """V3mTo2n[side*4+rel] (npts x B), V3mTo2nTWDivM (B x npts), resample (npts x npts), points, weights.

    rel 0 is the unrotated face (plus side); rel h >= 1 maps the points with orientation h - 1
    (minus side, faceRelation = sideOrientation + 1, DynamicRuptureMatrices.cpp:159-165).
    """
    pts, ws = stroud_points(order)
    ids = basis_indices3(order)
    mass = global_matrices(order)["M"]
    v3m, tw = [], []
    for side in range(4):
        for rel in range(4):
            chi, tau = pts[:, 0], pts[:, 1]
            if rel > 0:
                chi, tau = orientation_map(rel - 1, chi, tau)
            x, y, z = face_point(side, chi, tau)
            V = np.array([tet_dubiner(*t, x, y, z) for t in ids]).T
            v3m.append(V)
            tw.append((V * ws[:, None]).T / mass[:, None])
    ids2 = basis_indices2(order)
    V2 = np.array([tri_dubiner(*t, pts[:, 0], pts[:, 1]) for t in ids2]).T
    fm = (V2 * ws[:, None]).T @ V2
    res = V2 @ np.linalg.solve(fm, (V2 * ws[:, None]).T)
    return {"V3mTo2n": v3m, "V3mTo2nTWDivM": tw, "resample": res, "points": pts, "weights": ws}


def gauss_legendre_time(order, dt):
    """ShiftedGaussLegendre(order, 0, dt): points and weights on [0, dt]."""
    x, w = leggauss(order)
    return (x + 1) * dt / 2, w * dt / 2


def friction_delta_t(points):
    """FrictionSolver::computeDeltaT (FrictionSolver.cpp:20-37)."""
    d = np.empty(len(points))
    d[0] = points[0]
    d[1:] = np.diff(points)
    d[-1] += points[0]
    return d


def fault_face_data(coords, material, plus_face):
    """Per fault face: TinvT, flux solvers and impedances (DynamicRuptureMatrices.cpp:290-476).

    plus_face: [nf, 4] = (plus cell, plus side, minus cell, minus side).  The normal is the
    outward normal of the plus face, tangent1 its first edge (MeshReader.cpp:160-200).
    """
    nf = plus_face.shape[0]
    tinvt = np.zeros((nf, 9, 9))
    fsp = np.zeros((nf, 9, 9))
    fsm = np.zeros((nf, 9, 9))
    imp = np.zeros((nf, 7))
    for f in range(nf):
        pc, ps, mc, ms = plus_face[f]
        v = coords[pc]
        a, b, c = (v[k] for k in FACE2NODES[ps])
        nrm = np.cross(b - a, c - a)
        nrm /= np.linalg.norm(nrm)
        t1 = (b - a) / np.linalg.norm(b - a)
        t2 = np.cross(nrm, t1)
        T, Ti = rotation_matrices(nrm, t1, t2)
        tinvt[f] = Ti.T

        def area_vol(cell, side):
            w = coords[cell]
            aa, bb, cc = (w[k] for k in FACE2NODES[side])
            area = 0.5 * np.linalg.norm(np.cross(bb - aa, cc - aa))
            vol = abs(np.dot(w[3] - w[0], np.cross(w[1] - w[0], w[2] - w[0]))) / 6.0
            return area, vol

        ap, vp_ = area_vol(pc, ps)
        am, vm_ = area_vol(mc, ms)
        rp, mup, lp = material[pc]
        rm, mum, lm = material[mc]
        fsp[f] = (-2.0 * ap / (6.0 * vp_)) * coefficient_matrix_T(rp, mup, lp, 0) @ T.T
        fsm[f] = (2.0 * am / (6.0 * vm_)) * coefficient_matrix_T(rm, mum, lm, 0) @ T.T
        zp = rp * math.sqrt((lp + 2 * mup) / rp)
        zs = rp * math.sqrt(mup / rp)
        zpn = rm * math.sqrt((lm + 2 * mum) / rm)
        zsn = rm * math.sqrt(mum / rm)
        etap = 1.0 / (1.0 / zp + 1.0 / zpn)
        etas = 1.0 / (1.0 / zs + 1.0 / zsn)
        imp[f] = [zp, zs, zpn, zsn, etap, etas, 1.0 / zs + 1.0 / zsn]
    return {"TinvT": tinvt, "fluxSolverPlus": fsp, "fluxSolverMinus": fsm, "imp": imp}
