"""ctypes front-end of the C oracle (TEST INFRASTRUCTURE ONLY).

Arrays follow the layouts documented in oracle/oracle.c.  Per-cell 9x9 operators are
passed as numpy [.., q, p] arrays and converted here to column-major (q + 9 p).
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

from . import dg_setup

HERE = os.path.dirname(os.path.abspath(__file__))
_libs = {}


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib(dtype=np.float64):
    key = np.dtype(dtype).name
    if key not in _libs:
        path = os.path.join(HERE, "liboracle_f64.so" if key == "float64" else "liboracle_f32.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        for fn in ("oracle_ader", "oracle_taylor", "oracle_local", "oracle_neighbor", "oracle_steps"):
            getattr(L, fn).restype = None
        L.oracle_derivatives_size.restype = C.c_int
        _libs[key] = L
    return _libs[key]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def pack_globals(order):
    g = dg_setup.global_matrices(order)
    parts = []
    for name, cnt in (("kDivM", 3), ("kDivMT", 3), ("rDivM", 4), ("fMrT", 4), ("rT", 4), ("fP", 3)):
        for i in range(cnt):
            parts.append(np.asfortranarray(g[name][i]).ravel(order="F"))
    return np.ascontiguousarray(np.concatenate(parts), dtype=np.float64)


def colmajor_ops(a, dtype):
    """[..., q, p] -> contiguous [..., p, q] i.e. column-major 9x9 blocks."""
    return np.ascontiguousarray(np.swapaxes(a, -1, -2), dtype=dtype)


class Oracle:
    def __init__(self, order, dtype=np.float64):
        self.order = order
        self.dtype = np.dtype(dtype)
        self.L = lib(dtype)
        self.g = pack_globals(order)
        self.B = dg_setup.nbasis3(order)

    def ader(self, Q, star, coeffs, want_derivs=False):
        n = Q.shape[0]
        Q = np.ascontiguousarray(Q, dtype=self.dtype)
        I = np.zeros_like(Q)
        d = None
        if want_derivs:
            d = np.zeros((n, self.L.oracle_derivatives_size(self.order)), dtype=self.dtype)
        self.L.oracle_ader(self.order, C.c_int64(n), _p(self.g), _p(Q), _p(colmajor_ops(star, self.dtype)),
                           _p(np.ascontiguousarray(coeffs, dtype=np.float64)), _p(I), _p(d) if d is not None else None)
        return (I, d) if want_derivs else I

    def taylor(self, derivs, coeffs):
        n = derivs.shape[0]
        out = np.zeros((n, 9, self.B), dtype=self.dtype)
        self.L.oracle_taylor(self.order, C.c_int64(n), _p(np.ascontiguousarray(derivs, dtype=self.dtype)),
                             _p(np.ascontiguousarray(coeffs, dtype=np.float64)), _p(out))
        return out

    def local(self, Q, I, star, aplus, face_type=None):
        Q = np.array(Q, dtype=self.dtype, order="C")
        ft = None if face_type is None else np.ascontiguousarray(face_type, dtype=np.int8)
        self.L.oracle_local(self.order, C.c_int64(Q.shape[0]), _p(self.g), _p(np.ascontiguousarray(I, dtype=self.dtype)),
                            _p(colmajor_ops(star, self.dtype)), _p(colmajor_ops(aplus, self.dtype)),
                            _p(ft) if ft is not None else None, _p(Q))
        return Q

    def neighbor(self, Q, I, aminus, nb, side, orient, face_type=None):
        Q = np.array(Q, dtype=self.dtype, order="C")
        ft = None if face_type is None else np.ascontiguousarray(face_type, dtype=np.int8)
        self.L.oracle_neighbor(self.order, C.c_int64(Q.shape[0]), _p(self.g), _p(np.ascontiguousarray(I, dtype=self.dtype)),
                               _p(colmajor_ops(aminus, self.dtype)), _p(np.ascontiguousarray(nb, dtype=np.int32)),
                               _p(np.ascontiguousarray(side, dtype=np.int8)), _p(np.ascontiguousarray(orient, dtype=np.int8)),
                               _p(ft) if ft is not None else None, _p(Q))
        return Q

    def steps(self, Q, star, aplus, aminus, nb, side, orient, dt, nsteps, face_type=None):
        Q = np.array(Q, dtype=self.dtype, order="C")
        Iw = np.zeros_like(Q)
        ft = None if face_type is None else np.ascontiguousarray(face_type, dtype=np.int8)
        coeffs = dg_setup.taylor_integrate(self.order, 0.0, dt)
        self.L.oracle_steps(self.order, C.c_int64(Q.shape[0]), _p(self.g), _p(Q), _p(colmajor_ops(star, self.dtype)),
                            _p(colmajor_ops(aplus, self.dtype)), _p(colmajor_ops(aminus, self.dtype)),
                            _p(np.ascontiguousarray(nb, dtype=np.int32)), _p(np.ascontiguousarray(side, dtype=np.int8)),
                            _p(np.ascontiguousarray(orient, dtype=np.int8)), _p(ft) if ft is not None else None,
                            _p(np.ascontiguousarray(coeffs, dtype=np.float64)), C.c_int(nsteps), _p(Iw))
        return Q


# ---------------------------------------------------------------------------
# Dynamic rupture (oracle_dr.c)
# ---------------------------------------------------------------------------
class RSParamsC(C.Structure):
    _fields_ = [("f0", C.c_double), ("b", C.c_double), ("v0", C.c_double), ("l", C.c_double), ("muw", C.c_double),
                ("vw", C.c_double), ("newton_tol", C.c_double), ("state_tol", C.c_double), ("max_newton", C.c_int),
                ("max_outer", C.c_int)]



STATE_FIELDS = ("psi", "v1", "v2", "slip1", "slip2", "slip", "mu", "trac1", "trac2")


class DrAuxC(C.Structure):
    """oracle_dr_aux: fault time, nucleation, outputs and the slip-weakening fields."""
    _fields_ = [("time", C.c_double), ("t0", C.c_double), ("s0", C.c_double), ("nucleate", C.c_int),
                ("nuc", C.c_void_p), ("peak", C.c_void_p), ("trup", C.c_void_p), ("tdyn", C.c_void_p),
                ("law", C.c_int), ("healing", C.c_double), ("v_star", C.c_double), ("prakash_length", C.c_double),
                ("tp_exponent", C.c_double), ("mu_s", C.c_void_p), ("mu_d", C.c_void_p), ("d_c", C.c_void_p),
                ("cohesion", C.c_void_p), ("t_forced", C.c_void_p), ("reg", C.c_void_p),
                ("tp", C.c_int), ("tp_alpha", C.c_double), ("tp_rhoc", C.c_double), ("tp_lambda", C.c_double),
                ("tp_t0", C.c_double), ("tp_p0", C.c_double), ("tp_hw", C.c_void_p), ("tp_hyd", C.c_void_p),
                ("tp_theta", C.c_void_p), ("tp_sigma", C.c_void_p), ("tp_temp", C.c_void_p), ("tp_pres", C.c_void_p)]


AUX_ARRAYS = ("nuc", "peak", "trup", "tdyn", "mu_s", "mu_d", "d_c", "cohesion", "t_forced", "reg", "dir1", "dir2",
              "onset", "taus", "taur", "tp_hw", "tp_hyd", "tp_theta", "tp_sigma", "tp_temp", "tp_pres")


def _aux_struct(aux):
    """Builds DrAuxC from a dict (scalars: time, t0, s0, nucleate, law, healing, v_star,
    prakash_length, tp_exponent; float64 arrays [nf, npts], nuc [nf, 3, npts], converted in place)."""
    if aux is None:
        return None
    for k in AUX_ARRAYS:
        if aux.get(k) is not None:
            aux[k] = np.ascontiguousarray(aux[k], np.float64)
    ptr = lambda k: aux[k].ctypes.data if aux.get(k) is not None else None
    return DrAuxC(aux.get("time", 0.0), aux.get("t0", 0.0), aux.get("s0", 0.0), int(aux.get("nucleate", 0)),
                  ptr("nuc"), ptr("peak"), ptr("trup"), ptr("tdyn"), int(aux.get("law", 0)),
                  aux.get("healing", -1.0), aux.get("v_star", 0.0), aux.get("prakash_length", 1.0),
                  aux.get("tp_exponent", 1.0 / 3.0), ptr("mu_s"), ptr("mu_d"), ptr("d_c"), ptr("cohesion"),
                  ptr("t_forced"), ptr("reg"), int(aux.get("tp", 0)), aux.get("tp_alpha", 0.0), aux.get("tp_rhoc", 1.0),
                  aux.get("tp_lambda", 0.0), aux.get("tp_t0", 0.0), aux.get("tp_p0", 0.0), ptr("tp_hw"), ptr("tp_hyd"),
                  ptr("tp_theta"), ptr("tp_sigma"), ptr("tp_temp"), ptr("tp_pres"))


def dr_collocation(order, dt):
    """Time points, weights, friction sub-steps and collocation coefficients t_s^p / p!."""
    tp, tw = dg_setup.gauss_legendre_time(order, dt)
    coll = np.array([[t ** p / math.factorial(p) for p in range(order)] for t in tp])
    return tp, tw, dg_setup.friction_delta_t(tp), coll


class DROracle:
    """FP64 dynamic-rupture step of the oracle on a fault described by the product's face list."""

    def __init__(self, order, faces, params, dtype=np.float64):
        self.order = order
        self.L = lib(dtype)
        self.dtype = np.dtype(dtype)
        m = dg_setup.dr_matrices(order)
        self.npts = m["points"].shape[0]
        self.v3m = np.ascontiguousarray(np.stack([np.asfortranarray(v).ravel(order="F") for v in m["V3mTo2n"]]))
        self.tw = np.ascontiguousarray(np.stack([np.asfortranarray(v).ravel(order="F") for v in m["V3mTo2nTWDivM"]]))
        self.res = np.ascontiguousarray(np.asfortranarray(m["resample"]).ravel(order="F"))
        self.f = faces
        # rate-and-state constants (unused by the slip-weakening laws, which may pass {})
        self.P = RSParamsC(*[params.get(k, 0) for k in ("f0", "b", "v0", "l", "muw", "vw", "newton_tol", "state_tol",
                                                         "max_newton", "max_outer")])
        for fn in ("oracle_dr_interpolate", "oracle_dr_friction", "oracle_dr_friction_lsw", "oracle_dr_friction_isr",
                   "oracle_dr_nodal_flux", "oracle_dr_precompute"):
            getattr(self.L, fn).restype = None

    def interpolate(self, derivs_per_face, side, rel, coll):
        """derivs_per_face: [nf, dsize] derivatives of the cell on this side."""
        nf = derivs_per_face.shape[0]
        nts = coll.shape[0]
        out = np.zeros((nf, nts, 9, self.npts), self.dtype)
        idx = np.arange(nf, dtype=np.int32)
        tinvt = np.ascontiguousarray(np.swapaxes(self.f["TinvT"], -1, -2), np.float64)
        self.L.oracle_dr_interpolate(self.order, self.npts, nts, C.c_int64(nf),
                                     _p(np.ascontiguousarray(derivs_per_face, self.dtype)), _p(idx),
                                     _p(np.ascontiguousarray(side, np.int8)), _p(np.ascontiguousarray(rel, np.int8)),
                                     _p(tinvt), _p(self.v3m), _p(np.ascontiguousarray(coll, np.float64)), _p(out))
        return out

    def friction(self, qip, qim, state, a, init, deltat, tweights, mlp=None, record=None, first_iters=None,
                 aux=None):
        """Updates state (dict of [nf, npts] float64 arrays) in place; returns imposed states and iterations.

        init [nf, 3, npts] (sn0, tau1_0, tau2_0) changes in place under nucleation; aux: optional
        dict of the fault time, nucleation and outputs (_aux_struct).

        record: optional [cap, 6] float32 array with a one-element int64 counter, (rec, count),
        receiving the samples of plainly started, converged first solves; first_iters: optional
        [nf, npts] int64 array accumulating the iterations of the first solve of each time point."""
        nf = qip.shape[0]
        nts = qip.shape[1]
        imp = np.ascontiguousarray(self.f["imp"][:, :7], np.float64)
        isp = np.zeros((nf, 9, self.npts), self.dtype)
        ism = np.zeros((nf, 9, self.npts), self.dtype)
        iters = np.zeros((nf, self.npts), np.int64)
        for k in STATE_FIELDS:
            state[k] = np.ascontiguousarray(state[k], np.float64)
        initc = np.ascontiguousarray(init, np.float64)
        ax = _aux_struct(aux)
        w = n = None
        if mlp is not None:
            w = np.ascontiguousarray(mlp[0], np.float32)
            n = np.ascontiguousarray(mlp[1], np.float32)
        self.L.oracle_dr_friction(self.npts, nts, C.c_int64(nf), C.byref(self.P), _p(imp),
                                  _p(np.ascontiguousarray(qip, self.dtype)), _p(np.ascontiguousarray(qim, self.dtype)),
                                  _p(np.ascontiguousarray(a, np.float64)), _p(initc),
                                  *[_p(state[k]) for k in STATE_FIELDS],
                                  _p(np.ascontiguousarray(deltat, np.float64)),
                                  _p(np.ascontiguousarray(tweights, np.float64)), _p(self.res), _p(isp), _p(ism),
                                  _p(iters), _p(w) if w is not None else None, _p(n) if n is not None else None,
                                  _p(first_iters) if first_iters is not None else None,
                                  _p(record[0]) if record is not None else None,
                                  C.c_int64(record[0].shape[0] if record is not None else 0),
                                  _p(record[1]) if record is not None else None,
                                  C.byref(ax) if ax is not None else None)
        if initc is not init:
            init[...] = initc
        return isp, ism, iters

    def friction_lsw(self, qip, qim, state, init, deltat, tweights, aux):
        """Linear slip weakening (aux["law"] 1, 2 or 3): updates state, init and the aux arrays in
        place; returns the imposed states."""
        nf = qip.shape[0]
        nts = qip.shape[1]
        imp = np.ascontiguousarray(self.f["imp"][:, :7], np.float64)
        isp = np.zeros((nf, 9, self.npts), self.dtype)
        ism = np.zeros((nf, 9, self.npts), self.dtype)
        for k in STATE_FIELDS:
            state[k] = np.ascontiguousarray(state[k], np.float64)
        initc = np.ascontiguousarray(init, np.float64)
        ax = _aux_struct(aux)
        self.L.oracle_dr_friction_lsw(self.npts, nts, C.c_int64(nf), _p(imp),
                                      _p(np.ascontiguousarray(qip, self.dtype)),
                                      _p(np.ascontiguousarray(qim, self.dtype)), _p(initc),
                                      *[_p(state[k]) for k in STATE_FIELDS[1:]],
                                      _p(np.ascontiguousarray(deltat, np.float64)),
                                      _p(np.ascontiguousarray(tweights, np.float64)), _p(self.res), _p(isp), _p(ism),
                                      C.byref(ax))
        if initc is not init:
            init[...] = initc
        return isp, ism

    def friction_isr(self, qip, qim, state, init, deltat, tweights, aux):
        """Imposed slip rates (aux["law"] 7, 8 or 9; aux arrays dir1, dir2, onset, taus, taur):
        updates state, init and the aux outputs in place; returns the imposed states."""
        nf = qip.shape[0]
        nts = qip.shape[1]
        imp = np.ascontiguousarray(self.f["imp"][:, :7], np.float64)
        isp = np.zeros((nf, 9, self.npts), self.dtype)
        ism = np.zeros((nf, 9, self.npts), self.dtype)
        for k in STATE_FIELDS:
            state[k] = np.ascontiguousarray(state[k], np.float64)
        initc = np.ascontiguousarray(init, np.float64)
        for k in ("dir1", "dir2", "onset", "taus", "taur"):
            aux[k] = np.ascontiguousarray(aux[k], np.float64)
        ax = _aux_struct(aux)
        self.L.oracle_dr_friction_isr(self.npts, nts, C.c_int64(nf), _p(imp),
                                      _p(np.ascontiguousarray(qip, self.dtype)),
                                      _p(np.ascontiguousarray(qim, self.dtype)), _p(initc),
                                      *[_p(state[k]) for k in ("v1", "v2", "slip1", "slip2", "slip", "trac1", "trac2")],
                                      _p(np.ascontiguousarray(deltat, np.float64)),
                                      _p(np.ascontiguousarray(tweights, np.float64)),
                                      *[_p(aux[k]) for k in ("dir1", "dir2", "onset", "taus", "taur")],
                                      _p(isp), _p(ism), C.byref(ax))
        if initc is not init:
            init[...] = initc
        return isp, ism

    def nodal_flux(self, Q, cells, side, rel, imposed, flux):
        Q = np.array(Q, dtype=self.dtype, order="C")
        fl = np.ascontiguousarray(np.swapaxes(flux, -1, -2), np.float64)
        self.L.oracle_dr_nodal_flux(self.order, self.npts, C.c_int64(cells.shape[0]),
                                    _p(np.ascontiguousarray(cells, np.int32)), _p(np.ascontiguousarray(side, np.int8)),
                                    _p(np.ascontiguousarray(rel, np.int8)), _p(self.tw),
                                    _p(np.ascontiguousarray(imposed, self.dtype)), _p(fl), _p(Q))
        return Q


def dr_full_step(o, dro, Q, cells, faces, state, a, init, dt, mlp=None, record=None, first_iters=None, aux=None):
    """One step of proxy kernel all_dr in FP64: ADER + local, fault, neighbour (the GPU's order).

    aux: fault time, nucleation, outputs and (law 1-3) the slip-weakening fields; its time
    advances by dt."""
    order = o.order
    ft = cells["face_type"]
    coeffs = dg_setup.taylor_integrate(order, 0.0, dt)
    star = cells["star"].astype(np.float64)
    I, d = o.ader(np.asarray(Q, np.float64), star, coeffs, want_derivs=True)
    Q = o.local(Q, I, star, cells["AplusT"].astype(np.float64), ft)
    tp, tw, deltat, coll = dr_collocation(order, dt)
    pc, mc = faces["cells"][:, 0], faces["cells"][:, 1]
    ps, ms, rel = faces["sides"][:, 0], faces["sides"][:, 1], faces["sides"][:, 2]
    qip = dro.interpolate(d[pc], ps, np.zeros_like(ps), coll)
    qim = dro.interpolate(d[mc], ms, rel, coll)
    if aux is not None and aux.get("law", 0) in (1, 2, 3):
        isp, ism = dro.friction_lsw(qip, qim, state, init, deltat, tw, aux)
        iters = np.zeros(state["v1"].shape, np.int64)
    elif aux is not None and aux.get("law", 0) in (7, 8, 9):
        isp, ism = dro.friction_isr(qip, qim, state, init, deltat, tw, aux)
        iters = np.zeros(state["v1"].shape, np.int64)
    else:
        isp, ism, iters = dro.friction(qip, qim, state, a, init, deltat, tw, mlp, record, first_iters, aux)
    if aux is not None:
        aux["time"] = aux.get("time", 0.0) + dt
    Q = dro.nodal_flux(Q, pc, ps, np.zeros_like(ps), isp, faces["fluxSolverPlus"])
    Q = dro.nodal_flux(Q, mc, ms, rel, ism, faces["fluxSolverMinus"])
    Q = o.neighbor(Q, I, cells["AminusT"].astype(np.float64), cells["neighbor"], cells["side"], cells["orient"], ft)
    return Q, isp, ism, iters, (d, qip, qim)


# ---------------------------------------------------------------------------
# Local time stepping, rate 2 (test infrastructure: FP64 restatement)
# ---------------------------------------------------------------------------

def lts_clusters(dt, neighbor, face_type, max_clusters, fault_cells=None):
    """Cluster k holds the cell time steps in [2^k dt0, 2^{k+1} dt0), capped at max_clusters - 1,
    then neighbouring clusters are lowered until they differ by at most one, and the two cells of
    every dynamic-rupture face (fault_cells [nf, 2]) share the lower cluster (maximum difference
    property, docs/local-timestepping.rst:91-96)."""
    dt = np.asarray(dt, np.float64)
    dt0 = dt.min()
    cl = np.clip(np.floor(np.log2(dt / dt0) + 1e-12).astype(np.int64), 0, max_clusters - 1)
    regular = np.asarray(face_type) == 0
    nb = np.asarray(neighbor)
    while True:
        lim = np.where(regular, cl[np.where(regular, nb, 0)] + 1, np.iinfo(np.int64).max).min(axis=1)
        new = np.minimum(cl, lim)
        if fault_cells is not None:
            pa, pb = fault_cells[:, 0], fault_cells[:, 1]
            m = np.minimum(new[pa], new[pb])
            new[pa] = m
            new[pb] = m
        if np.array_equal(new, cl):
            return cl, dt0
        cl = new


def _dr_cluster_step(o, dr, Q, derivs, fsel, dt, time=0.0):
    """The fault step of the faces fsel over one step dt of their cluster, from the derivatives
    stored at the start of that step (fault time `time`); updates dr["state"] (and dr["init"],
    dr["aux"]) in place and returns Q."""
    faces, params = dr["faces"], dr["params"]
    sub = {k: np.asarray(v)[fsel] for k, v in faces.items()}
    dro = DROracle(o.order, sub, params)
    state = {k: np.ascontiguousarray(v[fsel]) for k, v in dr["state"].items()}
    tp, tw, deltat, coll = dr_collocation(o.order, dt)
    pc, mc = sub["cells"][:, 0], sub["cells"][:, 1]
    ps, ms, rel = sub["sides"][:, 0], sub["sides"][:, 1], sub["sides"][:, 2]
    qip = dro.interpolate(derivs[pc], ps, np.zeros_like(ps), coll)
    qim = dro.interpolate(derivs[mc], ms, rel, coll)
    init = np.ascontiguousarray(dr["init"][fsel], np.float64)
    aux = None
    if dr.get("aux") is not None:
        aux = {k: (np.ascontiguousarray(v[fsel]) if k in AUX_ARRAYS and v is not None else v)
               for k, v in dr["aux"].items()}
        aux["time"] = time
    if aux is not None and aux.get("law", 0) in (1, 2, 3):
        isp, ism = dro.friction_lsw(qip, qim, state, init, deltat, tw, aux)
    elif aux is not None and aux.get("law", 0) in (7, 8, 9):
        isp, ism = dro.friction_isr(qip, qim, state, init, deltat, tw, aux)
    else:
        isp, ism, _ = dro.friction(qip, qim, state, dr["a"][fsel], init, deltat, tw, aux=aux)
    for k, v in state.items():
        dr["state"][k][fsel] = v
    dr["init"][fsel] = init
    if aux is not None:
        for k in AUX_ARRAYS:
            if dr["aux"].get(k) is not None:
                dr["aux"][k][fsel] = aux[k]
    Q = dro.nodal_flux(Q, pc, ps, np.zeros_like(ps), isp, sub["fluxSolverPlus"])
    return dro.nodal_flux(Q, mc, ms, rel, ism, sub["fluxSolverMinus"])


def lts_cycles(o, Q, cells, cluster, dt0, ncycles, dr=None, on_predict=None, on_correct=None):
    """Rate-2 LTS (TimeCluster.cpp:358-440, 695-717; TimeCommon.cpp:40-87) in FP64.

    dr (optional): {"faces", "params", "state", "a", "init"[, "aux"]} of a fault whose faces join
    their cells' cluster: each cluster's correction runs the fault step of its faces over its own
    time step before the neighbour flux (TimeCluster.cpp:804-823); dr["state"] is updated in
    place, and dr["aux"] (fault time at the cycle start, nucleation, outputs, slip-weakening
    fields) too, its time advancing by the cycle length.  on_predict(cluster, step start offset in
    the run, its time step, Q) is called before each cluster's predictor (receivers);
    on_correct(cells of the cluster, its time step, Q) after each cluster's neighbour flux
    (plasticity, TimeCluster.cpp:966-975), and may change Q in place.

    Every cycle advances all clusters by dt0 2^(C-1).  At sub-step k of the finest cluster the
    clusters whose step starts there predict (ADER with derivatives, integration buffer of cells
    with a coarser neighbour -- reset when the coarser step starts --, local integral); then the
    clusters whose step ends at k + 1 correct: each regular face takes the neighbour's I (same
    cluster), its buffer (finer) or the Taylor integral of its derivatives over this step's
    sub-interval of the neighbour's step (coarser)."""
    order = o.order
    Q = np.array(Q, dtype=np.float64)
    n = Q.shape[0]
    cluster = np.asarray(cluster)
    ncl = int(cluster.max()) + 1
    star, aplus, aminus = (cells[k].astype(np.float64) for k in ("star", "AplusT", "AminusT"))
    nb, side, orient, ft = cells["neighbor"], cells["side"], cells["orient"], cells["face_type"]
    I = np.zeros_like(Q)
    buf = np.zeros_like(Q)
    derivs = None
    regular = ft == 0
    ncl_of = np.where(regular, cluster[np.where(regular, nb, 0)], cluster[:, None])
    has_coarser = (regular & (ncl_of > cluster[:, None])).any(axis=1)
    steps = 1 << (ncl - 1)
    for cyc in range(ncycles):
        for k in range(steps):
            for c in range(ncl):
                ln = 1 << c
                if k % ln:
                    continue
                idx = np.nonzero(cluster == c)[0]
                if idx.size == 0:
                    continue
                if on_predict is not None:
                    on_predict(c, (cyc * steps + k) * dt0, ln * dt0, Q)
                Ic, d = o.ader(Q[idx], star[idx], dg_setup.taylor_integrate(order, 0.0, dt0 * ln), want_derivs=True)
                I[idx] = Ic
                if derivs is None:
                    derivs = np.zeros((n, d.shape[1]))
                derivs[idx] = d
                b = idx[has_coarser[idx]]
                if (k // ln) % 2 == 0:
                    buf[b] = I[b]
                else:
                    buf[b] += I[b]
                Q[idx] = o.local(Q[idx], I[idx], star[idx], aplus[idx], ft[idx])
            for c in range(ncl):
                ln = 1 << c
                if (k + 1) % ln:
                    continue
                idx = np.nonzero(cluster == c)[0]
                if idx.size == 0:
                    continue
                a = ((k + 1 - ln) % (2 * ln)) * dt0
                sub = dg_setup.taylor_integrate(order, a, a + ln * dt0)
                faces = np.zeros((idx.size, 4) + Q.shape[1:])
                for f in range(4):
                    nbs = nb[idx, f]
                    reg = regular[idx, f]
                    ncf = np.where(reg, cluster[np.where(reg, nbs, 0)], c)
                    same, finer, coarser = reg & (ncf == c), reg & (ncf < c), reg & (ncf > c)
                    faces[same, f] = I[nbs[same]]
                    faces[finer, f] = buf[nbs[finer]]
                    if coarser.any():
                        faces[coarser, f] = o.taylor(derivs[nbs[coarser]], sub)
                pool = faces.reshape((-1,) + Q.shape[1:])
                pidx = np.arange(idx.size * 4, dtype=np.int32).reshape(idx.size, 4)
                if dr is not None:
                    fsel = np.nonzero(cluster[dr["faces"]["cells"][:, 0]] == c)[0]
                    if fsel.size:
                        t = dr["aux"].get("time", 0.0) + (k + 1 - ln) * dt0 if dr.get("aux") is not None else 0.0
                        Q = _dr_cluster_step(o, dr, Q, derivs, fsel, dt0 * ln, t)
                Q[idx] = o.neighbor(Q[idx], pool, aminus[idx], pidx, side[idx], orient[idx], ft[idx])
                if on_correct is not None:
                    on_correct(idx, ln * dt0, Q)
        if dr is not None and dr.get("aux") is not None:
            dr["aux"]["time"] = dr["aux"].get("time", 0.0) + steps * dt0
    return Q
