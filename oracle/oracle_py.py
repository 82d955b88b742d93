"""ctypes front-end of the C oracle (TEST INFRASTRUCTURE ONLY).

Arrays follow the layouts documented in oracle/oracle.c.  Per-cell 9x9 operators are
passed as numpy [.., q, p] arrays and converted here to column-major (q + 9 p).
"""
import ctypes as C
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
