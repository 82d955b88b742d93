"""Test infrastructure: FP64 numpy restatement of the viscoelastic element update (9 elastic
quantities + 6 memory variables for each of 3 mechanisms = 27 quantities), the checker of the GPU
viscoelastic kernels.  Dense 27 x 27 operators, exactly as the reference's equations define them:

* attenuation fit                 src/Physics/Attenuation.h:24-104
* A^T with anelastic coupling     src/Equations/viscoelastic/Model/ViscoelasticSetup.h:26-93
* source matrix E^T               ViscoelasticSetup.h:51-81
* face rotation (memory blocks)   ViscoelasticSetup.h:117-131
* flux solvers                    codegen/kernels/aderdg.py:226-246 (Godunov state of the elastic part)
* ADER with source term           codegen/kernels/aderdg.py:463-537 (dQ_i = dQ_{i-1} E + sum_d kDivMT_d dQ_{i-1} star_d)
* volume + local flux             codegen/kernels/aderdg.py:321-386 (Q += sum_d kDivM_d I star_d + I E + flux)
* neighbour flux                  codegen/kernels/aderdg.py:414-428

Arrays: Q [n][27][B] (quantity, then basis); quantities 0..8 elastic (sxx, syy, szz, sxy, syz,
sxz, u, v, w), 9 + 6 m + j memory variable j of mechanism m.
"""
import math

import numpy as np

from . import dg_setup

NMECH = 3
NQ = 9 + 6 * NMECH


def fit_attenuation(rho, mu, lam, qp, qs, freq_central, freq_ratio, nmech=NMECH):
    """Unrelaxed mu, lambda, relaxation frequencies omega [nmech] and theta [nmech][3]."""
    kmax = 2 * nmech - 1
    w0 = 2 * math.pi * freq_central
    wmin = w0 / math.sqrt(freq_ratio)
    if nmech > 1:
        w = np.exp(math.log(wmin) + np.arange(kmax) / (kmax - 1) * math.log(freq_ratio))
    else:
        w = np.array([w0])
    omega = w[0::2][:nmech].copy()
    wj = w[0::2][:nmech]
    norm = wj[None, :] ** 2 + w[:, None] ** 2
    sc1 = wj[None, :] * w[:, None]
    ap = (sc1 + wj[None, :] ** 2 / qp) / norm
    as_ = (sc1 + wj[None, :] ** 2 / qs) / norm
    alpha = np.linalg.lstsq(ap, np.full(kmax, 1.0 / qp), rcond=None)[0]
    beta = np.linalg.lstsq(as_, np.full(kmax, 1.0 / qs), rcond=None)[0]
    r = w0 / wj
    d = 1 + r * r
    psi1p, psi2p = 1 - (alpha / d).sum(), (alpha * r / d).sum()
    psi1s, psi2s = 1 - (beta / d).sum(), (beta * r / d).sum()
    rp = math.hypot(psi1p, psi2p)
    var_p = (lam + 2 * mu) * (rp + psi1p) / (2 * rp * rp)
    rs = math.hypot(psi1s, psi2s)
    var_mu = mu * (rs + psi1s) / (2 * rs * rs)
    t1 = -var_p * alpha
    t2 = -2.0 * var_mu * beta
    theta = np.stack([t1, t1 - t2, t2], axis=1)
    return var_mu, var_p - 2 * var_mu, omega, theta


def coefficient_matrix_T(rho, mu, lam, omega, dim):
    a = np.zeros((NQ, NQ))
    a[:9, :9] = dg_setup.coefficient_matrix_T(rho, mu, lam, dim)
    for m, om in enumerate(omega):
        col = 9 + 6 * m
        if dim == 0:
            a[6, col], a[7, col + 3], a[8, col + 5] = -om, -0.5 * om, -0.5 * om
        elif dim == 1:
            a[7, col + 1], a[6, col + 3], a[8, col + 4] = -om, -0.5 * om, -0.5 * om
        else:
            a[8, col + 2], a[7, col + 4], a[6, col + 5] = -om, -0.5 * om, -0.5 * om
    return a


def source_matrix_T(omega, theta):
    e = np.zeros((NQ, NQ))
    for m in range(len(omega)):
        o = 9 + 6 * m
        t0, t1, t2 = theta[m]
        e[o, 0], e[o + 1, 0], e[o + 2, 0] = t0, t1, t1
        e[o, 1], e[o + 1, 1], e[o + 2, 1] = t1, t0, t1
        e[o, 2], e[o + 1, 2], e[o + 2, 2] = t1, t1, t0
        e[o + 3, 3] = e[o + 4, 4] = e[o + 5, 5] = t2
        for i in range(6):
            e[o + i, o + i] = -omega[m]
    return e


def rotation_matrices(n, s, t):
    T9, Ti9 = dg_setup.rotation_matrices(n, s, t)
    T, Ti = np.zeros((NQ, NQ)), np.zeros((NQ, NQ))
    T[:9, :9], Ti[:9, :9] = T9, Ti9
    for m in range(NMECH):
        o = 9 + 6 * m
        T[o:o + 6, o:o + 6] = T9[:6, :6]
        Ti[o:o + 6, o:o + 6] = Ti9[:6, :6]
    return T, Ti


def cell_operators(coords, material, omega, theta, neighbor):
    """material [n][3] = rho and the unrelaxed mu, lambda; theta [n][3][3].  Returns star
    [n][3][27][27], ET [n][27][27], AplusT / AminusT [n][4][27][27] (numpy [q, p] = view (q, p))."""
    n = coords.shape[0]
    star = np.zeros((n, 3, NQ, NQ))
    et = np.zeros((n, NQ, NQ))
    ap = np.zeros((n, 4, NQ, NQ))
    am = np.zeros((n, 4, NQ, NQ))
    for c in range(n):
        rho, mu, lam = material[c]
        At = [coefficient_matrix_T(rho, mu, lam, omega, d) for d in range(3)]
        x, y, z = coords[c, :, 0], coords[c, :, 1], coords[c, :, 2]
        grads = dg_setup.reference_jacobian(x, y, z)
        for e in range(3):
            star[c, e] = grads[e][0] * At[0] + grads[e][1] * At[1] + grads[e][2] * At[2]
        et[c] = source_matrix_T(omega, theta[c])
        v = coords[c]
        vol = abs(np.dot(v[3] - v[0], np.cross(v[1] - v[0], v[2] - v[0]))) / 6.0
        for f in range(4):
            a, b, cc = (v[k] for k in dg_setup.FACE2NODES[f])
            nrm = np.cross(b - a, cc - a)
            area = 0.5 * np.linalg.norm(nrm)
            t1 = b - a
            t2 = np.cross(nrm, t1)
            nrm, t1, t2 = nrm / np.linalg.norm(nrm), t1 / np.linalg.norm(t1), t2 / np.linalg.norm(t2)
            nbm = material[neighbor[c, f]] if neighbor[c, f] >= 0 else material[c]
            g9l, g9n = dg_setup.godunov_state(material[c], nbm)
            gl, gn = np.zeros((NQ, NQ)), np.zeros((NQ, NQ))
            gl[:9, :9], gn[:9, :9] = g9l, g9n
            T, Ti = rotation_matrices(nrm, t1, t2)
            scale = -2.0 * area / (6.0 * vol)
            atil = coefficient_matrix_T(rho, mu, lam, omega, 0)  # isotropic: face-aligned A~^T = A^T
            ap[c, f] = scale * Ti.T @ (gl @ atil) @ T.T
            am[c, f] = scale * Ti.T @ (gn @ atil) @ T.T
    return {"star": star, "ET": et, "AplusT": ap, "AminusT": am}


class Visco:
    """Dense FP64 viscoelastic element update at one convergence order."""

    def __init__(self, order):
        self.order = order
        g = dg_setup.global_matrices(order)
        self.kdm = np.stack(g["kDivM"])
        self.kdmt = np.stack(g["kDivMT"])
        self.rdivm, self.fmrt, self.rt, self.fp = g["rDivM"], g["fMrT"], g["rT"], g["fP"]
        self.flux = np.stack([self.rdivm[f] @ self.fmrt[f] for f in range(4)])

    def ader(self, Q, star, et, dt):
        """Time-integrated DOFs over [0, dt] (source term keeps all basis rows at every stage)."""
        c = dg_setup.taylor_integrate(self.order, 0.0, dt)
        dq = np.array(Q, dtype=np.float64)
        I = c[0] * dq
        for i in range(1, self.order):
            t = np.einsum("dkl,nql->ndqk", self.kdmt, dq)
            dq = np.einsum("ndqk,ndqp->npk", t, star) + np.einsum("nqk,nqp->npk", dq, et)
            I = I + c[i] * dq
        return I

    def local(self, Q, I, star, et, aplus, face_type):
        vol = np.einsum("dkl,nql,ndqp->npk", self.kdm, I, star) + np.einsum("nqk,nqp->npk", I, et)
        ap = np.where((face_type == 1)[:, :, None, None], 0.0, aplus)
        flux = np.einsum("fkl,nql,nfqp->npk", self.flux, I, ap)
        return Q + vol + flux

    def neighbor(self, Q, I, aminus, nb, side, orient, face_type):
        Q = np.array(Q, dtype=np.float64)
        F = self.fp[0].shape[0]
        for f in range(4):
            on = (face_type[:, f] == 0) & (nb[:, f] >= 0)
            t1 = np.zeros((Q.shape[0], NQ, F))
            for j in range(4):
                m = on & (side[:, f] == j)
                t1[m] = np.einsum("ml,nql->nqm", self.rt[j], I[nb[m, f]])
            t2 = np.zeros_like(t1)
            for h in range(3):
                m = on & (orient[:, f] == h)
                t2[m] = np.einsum("ab,nqb->nqa", self.fp[h], t1[m])
            t3 = np.einsum("nqm,nqp->npm", t2, aminus[:, f])
            Q[on] += np.einsum("km,npm->npk", self.rdivm[f], t3[on])
        return Q

    def steps(self, Q, ops, nb, side, orient, face_type, dt, nsteps):
        Q = np.array(Q, dtype=np.float64)
        for _ in range(nsteps):
            I = self.ader(Q, ops["star"], ops["ET"], dt)
            Q = self.local(Q, I, ops["star"], ops["ET"], ops["AplusT"], face_type)
            Q = self.neighbor(Q, I, ops["AminusT"], nb, side, orient, face_type)
        return Q


class ViscoLts:
    """The dense viscoelastic update behind the interface of the elastic oracle that
    oracle_py.lts_cycles drives: ader with Taylor coefficients and derivatives, local, neighbour and
    taylor.  Its star argument carries the three star matrices and the source matrix ET as
    star[:, 0:3] and star[:, 3] ([n, 4, 27, 27]); derivatives are [n, order * 27 * B], stage-major,
    with all basis rows at every stage (the source term keeps them, aderdg.py:507-517)."""

    def __init__(self, order):
        self.order = order
        self.v = Visco(order)

    def ader(self, Q, star, coeffs, want_derivs=False):
        dq = np.array(Q, dtype=np.float64)
        I = coeffs[0] * dq
        ds = [dq]
        for i in range(1, self.order):
            t = np.einsum("dkl,nql->ndqk", self.v.kdmt, dq)
            dq = np.einsum("ndqk,ndqp->npk", t, star[:, :3]) + np.einsum("nqk,nqp->npk", dq, star[:, 3])
            I = I + coeffs[i] * dq
            ds.append(dq)
        if not want_derivs:
            return I
        return I, np.stack(ds, axis=1).reshape(dq.shape[0], -1)

    def taylor(self, derivs, coeffs):
        n = derivs.shape[0]
        d = derivs.reshape(n, self.order, NQ, -1)
        return np.einsum("i,niqk->nqk", np.asarray(coeffs[:self.order], np.float64), d)

    def local(self, Q, I, star, aplus, face_type=None):
        return self.v.local(Q, I, star[:, :3], star[:, 3], aplus, face_type)

    def neighbor(self, Q, I, aminus, nb, side, orient, face_type=None):
        return self.v.neighbor(Q, I, aminus, nb, side, orient, face_type)
