"""Global ADER-DG matrices of the reference, derived by exact polynomial integration.

The modal basis is the reference's Dubiner basis on the unit tetrahedron
(src/Numerical/Functions.cpp:63-160, ordering src/Numerical/BasisFunction.h:133-142).
Each basis polynomial is expanded into monomials xi^a eta^b zeta^c and all integrals are
evaluated in closed form (int_tet xi^a eta^b zeta^c = a! b! c! / (a+b+c+3)!), so the
matrices carry no quadrature error.  The matrices match the reference's
codegen/matrices/matrices_{20,35,56}.xml, the names follow codegen/kernels/aderdg.py:

    kDivM[d]  = M^-1 K_d,  K_d[k,l] = int dphi_k/dxi_d phi_l
    kDivMT[d] = -M^-1 K_d^T (sign applied at load in src/Memory/GlobalData.cpp:51-61)
    rT[f]     face-f trace of phi_l in the face basis psi_n (projection coefficients)
    fMrT[f]   = fM rT[f] (fM = face mass, diagonal)
    rDivM[f]  = M^-1 rT[f]^T
    fP[h]     = int psi_m(chi, tau) psi_n(map_h(chi, tau)) over the face triangle
"""
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache

import numpy as np

FACE2NODES = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (1, 2, 3))


def nb3(order: int) -> int:
    return order * (order + 1) * (order + 2) // 6


def nb2(order: int) -> int:
    return order * (order + 1) // 2


class Poly:
    """Sparse polynomial in nv variables with exact rational coefficients."""

    __slots__ = ("nv", "t")

    def __init__(self, nv, terms=None):
        self.nv = nv
        self.t = dict(terms or {})

    @staticmethod
    def const(nv, c):
        return Poly(nv, {(0,) * nv: Fraction(c)})

    @staticmethod
    def var(nv, i, scale=1, shift=0):
        e = [0] * nv
        e[i] = 1
        p = Poly(nv, {tuple(e): Fraction(scale)})
        if shift:
            p.t[(0,) * nv] = Fraction(shift)
        return p

    def __add__(self, o):
        if not isinstance(o, Poly):
            o = Poly.const(self.nv, o)
        r = dict(self.t)
        for k, v in o.t.items():
            r[k] = r.get(k, 0) + v
        return Poly(self.nv, {k: v for k, v in r.items() if v != 0})

    __radd__ = __add__

    def __neg__(self):
        return Poly(self.nv, {k: -v for k, v in self.t.items()})

    def __sub__(self, o):
        return self + (-o if isinstance(o, Poly) else -Fraction(o))

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        if not isinstance(o, Poly):
            o = Fraction(o)
            return Poly(self.nv, {k: v * o for k, v in self.t.items() if v * o != 0})
        r = {}
        for k1, v1 in self.t.items():
            for k2, v2 in o.t.items():
                k = tuple(a + b for a, b in zip(k1, k2))
                r[k] = r.get(k, 0) + v1 * v2
        return Poly(self.nv, {k: v for k, v in r.items() if v != 0})

    __rmul__ = __mul__

    def deriv(self, i):
        r = {}
        for k, v in self.t.items():
            if k[i] > 0:
                kk = list(k)
                kk[i] -= 1
                r[tuple(kk)] = r.get(tuple(kk), 0) + v * k[i]
        return Poly(self.nv, r)

    def compose(self, subs):
        """Substitute variable i by polynomial subs[i] (all in a common target space)."""
        nv2 = subs[0].nv
        out = Poly(nv2)
        cache = {}
        for k, v in self.t.items():
            term = Poly.const(nv2, v)
            for i, e in enumerate(k):
                if e:
                    key = (i, e)
                    if key not in cache:
                        p = Poly.const(nv2, 1)
                        for _ in range(e):
                            p = p * subs[i]
                        cache[key] = p
                    term = term * cache[key]
            out = out + term
        return out


def _sf_jacobi(n, a, b, x: Poly, y: Poly) -> Poly:
    """y^n P_n^{(a,b)}(x/y) as a polynomial (three-term recurrence, Functions.cpp:63-76)."""
    nv = x.nv
    if n == 0:
        return Poly.const(nv, 1)
    pm1 = Poly.const(nv, 1)
    pm = y * Fraction(a - b, 2) + x * (1 + Fraction(a + b, 2))
    for m in range(2, n + 1):
        pm2, pm1 = pm1, pm
        c0 = 2 * m + a + b
        pm = ((y * Fraction(a * a - b * b) + x * Fraction(c0 * (c0 - 2))) * pm1 * Fraction(c0 - 1)
              - y * y * pm2 * Fraction(2 * (m + a - 1) * (m + b - 1) * c0)) * Fraction(1, 2 * m * (m + a + b) * (c0 - 2))
    return pm


def tet_basis(order):
    xi, eta, zeta = (Poly.var(3, i) for i in range(3))
    one = Poly.const(3, 1)
    out = []
    for o in range(order):
        for k in range(o + 1):
            for j in range(o - k + 1):
                i = o - j - k
                out.append(_sf_jacobi(i, 0, 0, xi * 2 - 1 + eta + zeta, one - eta - zeta)
                           * _sf_jacobi(j, 2 * i + 1, 0, eta * 2 - 1 + zeta, one - zeta)
                           * _sf_jacobi(k, 2 * i + 2 * j + 2, 0, zeta * 2 - 1, one))
    return out


def tri_basis(order):
    x, y = Poly.var(2, 0), Poly.var(2, 1)
    one = Poly.const(2, 1)
    out = []
    for o in range(order):
        for j in range(o + 1):
            i = o - j
            out.append(_sf_jacobi(i, 0, 0, x * 2 - 1 + y, one - y) * _sf_jacobi(j, 2 * i + 1, 0, y * 2 - 1, one))
    return out


def _int_simplex(p: Poly) -> Fraction:
    """Exact integral over the unit simplex of dimension p.nv."""
    s = Fraction(0)
    d = p.nv
    for k, v in p.t.items():
        num = 1
        for e in k:
            num *= math.factorial(e)
        s += v * Fraction(num, math.factorial(sum(k) + d))
    return s


def _face_subs(face):
    """(chi, tau) -> (xi, eta, zeta) for face f (src/Numerical/Transformation.cpp:300-348)."""
    chi, tau = Poly.var(2, 0), Poly.var(2, 1)
    zero = Poly(2)
    one = Poly.const(2, 1)
    return {0: [tau, chi, zero], 1: [chi, zero, tau], 2: [zero, tau, chi], 3: [one - chi - tau, chi, tau]}[face]


def _orient_subs(h):
    chi, tau = Poly.var(2, 0), Poly.var(2, 1)
    one = Poly.const(2, 1)
    return {0: [tau, chi], 1: [one - chi - tau, tau], 2: [chi, one - chi - tau]}[h]


@lru_cache(maxsize=None)
def global_matrices(order: int) -> dict:
    phi = tet_basis(order)
    psi = tri_basis(order)
    B, F = len(phi), len(psi)
    mass = [_int_simplex(p * p) for p in phi]
    fmass = [_int_simplex(p * p) for p in psi]
    dphi = [[p.deriv(d) for p in phi] for d in range(3)]
    K = [[[_int_simplex(dphi[d][k] * phi[l]) for l in range(B)] for k in range(B)] for d in range(3)]
    kdivm = [np.array([[float(K[d][k][l] / mass[k]) for l in range(B)] for k in range(B)]) for d in range(3)]
    kdivmt = [np.array([[float(-K[d][l][k] / mass[k]) for l in range(B)] for k in range(B)]) for d in range(3)]
    rT, fMrT, rDivM = [], [], []
    for f in range(4):
        subs = _face_subs(f)
        traces = [p.compose(subs) for p in phi]
        S = [[_int_simplex(psi[n] * traces[l]) for l in range(B)] for n in range(F)]
        rT.append(np.array([[float(S[n][l] / fmass[n]) for l in range(B)] for n in range(F)]))
        fMrT.append(np.array([[float(S[n][l]) for l in range(B)] for n in range(F)]))
        rDivM.append(np.array([[float(S[n][k] / fmass[n] / mass[k]) for n in range(F)] for k in range(B)]))
    fP = []
    for h in range(3):
        subs = _orient_subs(h)
        psih = [p.compose(subs) for p in psi]
        fP.append(np.array([[float(_int_simplex(psi[m] * psih[n])) for n in range(F)] for m in range(F)]))
    return {"kDivM": kdivm, "kDivMT": kdivmt, "rT": rT, "fMrT": fMrT, "rDivM": rDivM, "fP": fP,
            "M": np.array([float(m) for m in mass]), "fM": np.array([float(m) for m in fmass])}


def _poly_eval(p: Poly, pts: np.ndarray) -> np.ndarray:
    """Evaluates a polynomial at points [n, nv]."""
    out = np.zeros(pts.shape[0])
    for k, v in p.t.items():
        term = np.full(pts.shape[0], float(v))
        for i, e in enumerate(k):
            if e:
                term = term * pts[:, i] ** e
        out += term
    return out


def _gauss_jacobi(n, alpha, beta):
    """Nodes and weights of Gauss-Jacobi on [-1, 1] by the Golub-Welsch eigenvalue method."""
    k = np.arange(n, dtype=float)
    ab = alpha + beta
    diag = np.empty(n)
    diag[0] = (beta - alpha) / (ab + 2)
    kk = k[1:]
    diag[1:] = (beta ** 2 - alpha ** 2) / ((2 * kk + ab) * (2 * kk + ab + 2))
    kk = np.arange(1, n, dtype=float)
    off = np.sqrt(4 * kk * (kk + alpha) * (kk + beta) * (kk + ab) / ((2 * kk + ab) ** 2 * (2 * kk + ab + 1) * (2 * kk + ab - 1)))
    J = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    x, vecs = np.linalg.eigh(J)
    mu0 = 2 ** (ab + 1) * math.gamma(alpha + 1) * math.gamma(beta + 1) / math.gamma(ab + 2)
    return x, mu0 * vecs[0] ** 2


def stroud_rule(order):
    """Conical-product points on the face triangle (order+1 per direction), the reference's ordering."""
    n = order + 1
    xj, wj = _gauss_jacobi(n, 1.0, 0.0)
    xl, wl = _gauss_jacobi(n, 0.0, 0.0)
    pts, ws = [], []
    for i in reversed(range(n)):
        u = (1 + xj[i]) / 2
        for j in range(n):
            pts.append((u, (1 - u) * (1 - xl[j]) / 2))
            ws.append(wj[i] / 4 * wl[j] / 2)
    return np.array(pts), np.array(ws)


@lru_cache(maxsize=None)
def dr_matrices(order: int) -> dict:
    """Dynamic-rupture face matrices (codegen/matrices/dr_stroud_matrices_{N}.json).

    V3mTo2n[side * 4 + rel]: 3D basis at the face quadrature points (npts x B); rel 0 is the
    plus side, rel >= 1 the minus side with orientation rel - 1.  V3mTo2nTWDivM = M^-1 V^T W.
    resample: L2 projection of point values onto the face basis, evaluated at the points.
    """
    pts, ws = stroud_rule(order)
    phi = tet_basis(order)
    psi = tri_basis(order)
    mass = np.array([float(_int_simplex(p * p)) for p in phi])
    v3m, tw = [], []
    for side in range(4):
        for rel in range(4):
            chi, tau = pts[:, 0], pts[:, 1]
            if rel == 1:
                chi, tau = tau, chi
            elif rel == 2:
                chi, tau = 1 - chi - tau, tau
            elif rel == 3:
                chi, tau = chi, 1 - chi - tau
            xyz = {0: (tau, chi, 0 * chi), 1: (chi, 0 * chi, tau), 2: (0 * chi, tau, chi),
                   3: (1 - chi - tau, chi, tau)}[side]
            P = np.stack(xyz, axis=1)
            V = np.stack([_poly_eval(p, P) for p in phi], axis=1)
            v3m.append(V)
            tw.append((V * ws[:, None]).T / mass[:, None])
    V2 = np.stack([_poly_eval(p, pts) for p in psi], axis=1)
    fm = (V2 * ws[:, None]).T @ V2
    res = V2 @ np.linalg.solve(fm, (V2 * ws[:, None]).T)
    return {"V3mTo2n": v3m, "V3mTo2nTWDivM": tw, "resample": res, "points": pts, "weights": ws}


def gauss_legendre01(n):
    """Gauss-Legendre nodes and weights on [0, 1]."""
    x, w = _gauss_jacobi(n, 0.0, 0.0)
    return (x + 1) / 2, w / 2
