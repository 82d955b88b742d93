"""ctypes bindings of libsei_gb300.so (C ABI in include/sei_gb300.h).

Numpy conventions used by this front-end: DOF tensors are [ncells, 9, B] (basis index
fastest, as the reference's column-major Q[k, p]); per-cell 9x9 operators are numpy arrays
indexed [..., q, p] (row q, column p of the reference's view) and are converted to the
ABI's column-major storage here.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsei_gb300.so")

SEI_OK = 0
ERRORS = {-1: "SEI_ERR_ARG", -2: "SEI_ERR_OOM", -3: "SEI_ERR_CUDA", -4: "SEI_ERR_TIMEOUT", -5: "SEI_ERR_NAN",
          -6: "SEI_ERR_STATE", -7: "SEI_ERR_UNSUPPORTED", -8: "SEI_ERR_CAPACITY"}
# Proxy kernel names (src/Proxy/Common.cpp:22-40) -> SEI_KERNEL_*.
KERNELS = {"all": 0, "local": 1, "neigh": 2, "ader": 3, "localwoader": 4, "neigh_dr": 5, "godunov_dr": 6, "all_dr": 7}


class SeiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Config(C.Structure):
    _fields_ = [("order", C.c_int), ("device", C.c_int), ("precision", C.c_int), ("store_derivatives", C.c_int)]


class _CubeParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double), ("rho", C.c_double),
                ("vp", C.c_double), ("vs", C.c_double), ("perturb", C.c_double), ("seed", C.c_uint64),
                ("fault_plane", C.c_int), ("grading", C.c_double), ("lts_profile", C.c_int)]


class RSParams(C.Structure):
    """sei_rs_params: fast-velocity-weakening rate-and-state friction and the seeded fault state."""
    _fields_ = [(n, C.c_double) for n in ("f0", "b", "v0", "l", "muw", "vw", "a_min", "a_max", "sn_min", "sn_max",
                                          "tau_min", "tau_max", "v_init", "newton_tol", "state_tol")] + \
               [("max_newton", C.c_int), ("max_outer", C.c_int), ("seed", C.c_uint64)]

    @classmethod
    def fault_config(cls, seed=7, **kw):
        """The rate-and-state set-up of the planar-fault workload (MPa as Pa)."""
        d = dict(f0=0.6, b=0.014, v0=1e-6, l=0.02, muw=0.1, vw=0.1, a_min=0.008, a_max=0.02, sn_min=-120e6,
                 sn_max=-40e6, tau_min=20e6, tau_max=75e6, v_init=1e-16, newton_tol=1e-8, state_tol=1e-8,
                 max_newton=60, max_outer=10, seed=seed)
        d.update(kw)
        return cls(**d)


class LSWParams(C.Structure):
    """sei_lsw_params: linear slip weakening (law 1), its bimaterial form (2) or the TP proxy (3)."""
    _fields_ = [("law", C.c_int)] + \
               [(n, C.c_double) for n in ("mu_s", "mu_d", "d_c", "cohesion", "sn_min", "sn_max", "tau_min", "tau_max",
                                          "forced_rupture_time", "t0", "healing_threshold", "v_star",
                                          "prakash_length", "tp_proxy_exponent")] + [("seed", C.c_uint64)]

    @classmethod
    def fault_config(cls, law=1, seed=7, **kw):
        """Slip-weakening set-up of the planar-fault workload: mu_s 0.677, mu_d 0.525 and stresses near
        those of the SCEC TPV5 benchmark (sn0 ~ U[-125, -115] MPa, tau1_0 ~ U[62, 78] MPa, below the
        static strength), d_c 0.01 m so that weakening completes within a few steps of 100 m cells,
        no forced rupture (set SEI_DR_FORCED_RUPTURE_TIME per point), no healing."""
        d = dict(law=law, mu_s=0.677, mu_d=0.525, d_c=0.01, cohesion=0.0, sn_min=-125e6, sn_max=-115e6,
                 tau_min=62e6, tau_max=78e6, forced_rupture_time=1e300, t0=0.0, healing_threshold=-1.0,
                 v_star=0.1, prakash_length=1.0, tp_proxy_exponent=1.0 / 3.0, seed=seed)
        d.update(kw)
        return cls(**d)


class TPParams(C.Structure):
    """sei_tp_params: thermal pressurisation of the rate-and-state laws."""
    _fields_ = [(n, C.c_double) for n in ("thermal_diffusivity", "heat_capacity", "undrained_tp_response",
                                          "initial_temperature", "initial_pressure", "half_width_shear_zone",
                                          "hydraulic_diffusivity")]


class ISRParams(C.Structure):
    """sei_isr_params: imposed slip rate, law 7 (regularised Yoffe), 8 (Gaussian) or 9 (delta)."""
    _fields_ = [("law", C.c_int)] + [(n, C.c_double) for n in ("slip_dir1", "slip_dir2", "onset_time", "tau_s", "tau_r",
                                                                "sn0", "tau1_0")]


DR_FIELDS = {"psi": 0, "slip_rate1": 1, "slip_rate2": 2, "slip1": 3, "slip2": 4, "slip": 5, "mu": 6, "traction1": 7,
             "traction2": 8, "a": 9, "sn0": 10, "tau1_0": 11, "tau2_0": 12, "mu_s": 13, "mu_d": 14, "d_c": 15,
             "cohesion": 16, "forced_rupture_time": 17, "peak_slip_rate": 18, "rupture_time": 19,
             "dyn_stress_time": 20, "nuc_sn": 21, "nuc_tau1": 22, "nuc_tau2": 23, "reg_strength": 24,
             "slip_dir1": 25, "slip_dir2": 26, "onset_time": 27, "tau_s": 28, "tau_r": 29, "tp_half_width": 30,
             "tp_hydraulic_diffusivity": 31, "tp_temperature": 32, "tp_pressure": 33}


class _Mesh(C.Structure):
    _fields_ = [("nvertices", C.c_int64), ("geometry", C.c_void_p), ("ncells", C.c_int64), ("connect", C.c_void_p),
                ("boundary", C.c_void_p), ("boundary_format", C.c_int), ("identify", C.c_void_p),
                ("material", C.c_void_p), ("fault_ref", C.c_double * 3), ("fault_ref_method", C.c_int)]


BOUNDARY_FORMATS = {"i32": 0, "i64": 1, "i32x4": 2}
FAULT_REF_METHODS = {"point": 0, "normal": 1}


class _Perf(C.Structure):
    _fields_ = [("nonzero_flop", C.c_double), ("hardware_flop", C.c_double), ("bytes", C.c_double)]


class _Tune(C.Structure):
    _fields_ = [("fused_local", C.c_int), ("tc_local", C.c_int), ("nb_ctas", C.c_int), ("nb_form", C.c_int),
                ("candidates", C.c_int),
                ("best_ms", C.c_double), ("worst_ms", C.c_double)]


_lib = None
VP = C.c_void_p


def _sig(lib, name, res, args):
    fn = getattr(lib, name)
    fn.restype = res
    fn.argtypes = args


def load_library(path: str | None = None):
    """Loads the CUDA library; raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise SeiError(-7, f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    i, i64, d = C.c_int, C.c_int64, C.c_double
    _sig(lib, "sei_version", i, [])
    _sig(lib, "sei_create", i, [C.POINTER(_Config), C.POINTER(VP)])
    _sig(lib, "sei_destroy", None, [VP])
    _sig(lib, "sei_last_error", C.c_char_p, [VP])
    _sig(lib, "sei_build_periodic_cube", i, [VP, C.POINTER(_CubeParams), C.POINTER(i64)])
    _sig(lib, "sei_set_cells", i, [VP, i64, VP, VP, VP, VP, VP, VP, VP])
    _sig(lib, "sei_num_cells", i64, [VP])
    _sig(lib, "sei_get_cells", i, [VP, VP, VP, VP, VP, VP, VP, VP])
    _sig(lib, "sei_get_geometry", i, [VP, VP, VP, VP])
    _sig(lib, "sei_cfl_timestep", i, [VP, d, C.POINTER(d)])
    _sig(lib, "sei_set_dofs", i, [VP, VP])
    _sig(lib, "sei_get_dofs", i, [VP, VP])
    _sig(lib, "sei_get_time_integrated", i, [VP, VP])
    _sig(lib, "sei_get_derivatives", i, [VP, VP])
    _sig(lib, "sei_derivatives_size", i, [i])
    _sig(lib, "sei_compute_ader", i, [VP, VP, d])
    _sig(lib, "sei_compute_local_integral", i, [VP])
    _sig(lib, "sei_compute_ader_local", i, [VP, d])
    _sig(lib, "sei_compute_neighbors_integral", i, [VP])
    _sig(lib, "sei_evaluate_taylor", i, [VP, VP, VP])
    _sig(lib, "sei_run", i, [VP, i, d, i])
    _sig(lib, "sei_run_host", i, [VP, i, d, i, VP, VP])
    _sig(lib, "sei_sync", i, [VP])
    _sig(lib, "sei_last_run_ms", i, [VP, C.POINTER(d)])
    _sig(lib, "sei_metrics", i, [VP, i, C.POINTER(_Perf)])
    _sig(lib, "sei_autotune", i, [VP, d, i, C.POINTER(_Tune)])
    _sig(lib, "sei_set_profiling", i, [VP, i])
    _sig(lib, "sei_set_option", i, [VP, i, i])
    _sig(lib, "sei_get_option", i, [VP, i, C.POINTER(i)])
    _sig(lib, "sei_tc_gemm_check", i, [VP, VP, VP, i, i, i])
    _sig(lib, "sei_tc_layout_check", i, [VP, VP, VP, i, i, i, i, i, i])
    _sig(lib, "sei_check_wait_timeout", i, [VP, i, i])
    _sig(lib, "sei_tc_ld_probe", i, [i, VP])
    _sig(lib, "sei_device_clock_khz", i, [i, C.POINTER(C.c_int)])
    _sig(lib, "sei_dr_setup", i, [VP, C.POINTER(RSParams), C.POINTER(i64)])
    _sig(lib, "sei_dr_setup_lsw", i, [VP, C.POINTER(LSWParams), C.POINTER(i64)])
    _sig(lib, "sei_dr_setup_rate_state", i, [VP, C.POINTER(RSParams), i, C.POINTER(i64)])
    _sig(lib, "sei_dr_setup_imposed", i, [VP, C.POINTER(ISRParams), C.POINTER(i64)])
    _sig(lib, "sei_dr_set_thermal_pressurization", i, [VP, i, C.POINTER(TPParams)])
    _sig(lib, "sei_set_mesh", i, [VP, C.POINTER(_Mesh), C.POINTER(i64), C.POINTER(i64)])
    _sig(lib, "sei_receivers_setup", i, [VP, i64, VP, C.c_double, C.c_uint, i, VP])
    _sig(lib, "sei_receivers_columns", i, [VP])
    _sig(lib, "sei_basis_functions", i, [i, VP, VP, VP])
    _sig(lib, "sei_receivers_read", i, [VP, VP, i64, C.POINTER(i64)])
    _sig(lib, "sei_plasticity_setup", i, [VP, VP, d, VP, VP, VP, i])
    _sig(lib, "sei_plasticity_disable", i, [VP])
    _sig(lib, "sei_plasticity_get_strain", i, [VP, VP])
    _sig(lib, "sei_plasticity_yield_count", i, [VP, C.POINTER(i64)])
    _sig(lib, "sei_plasticity_relax_factor", d, [d, d])
    _sig(lib, "sei_plasticity_nodes", i, [i, VP])
    _sig(lib, "sei_get_time", i, [VP, C.POINTER(C.c_double)])
    _sig(lib, "sei_set_time", i, [VP, C.c_double])
    _sig(lib, "sei_fault_output_setup", i, [VP, i, VP, i])
    _sig(lib, "sei_fault_output_read", i, [VP, VP, i64, C.POINTER(i64)])
    _sig(lib, "sei_dr_law", i, [VP])
    _sig(lib, "sei_dr_set_nucleation", i, [VP, i, C.c_double, C.c_double])
    _sig(lib, "sei_dr_get_time", i, [VP, C.POINTER(C.c_double)])
    _sig(lib, "sei_dr_set_time", i, [VP, C.c_double])
    _sig(lib, "sei_dr_num_points", i, [i])
    _sig(lib, "sei_dr_num_faces", i64, [VP])
    _sig(lib, "sei_dr_get_faces", i, [VP, VP, VP, VP, VP, VP, VP])
    _sig(lib, "sei_dr_get_state", i, [VP, i, VP])
    _sig(lib, "sei_dr_set_state", i, [VP, i, VP])
    _sig(lib, "sei_dr_get_imposed", i, [VP, VP, VP])
    _sig(lib, "sei_dr_newton_iterations", i, [VP, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)])
    _sig(lib, "sei_dr_newton_iterations32", i, [VP, C.POINTER(i64)])
    _sig(lib, "sei_dr_reset_counters", i, [VP])
    _sig(lib, "sei_dr_faces_step", i, [VP, d])
    _sig(lib, "sei_dr_get_slots", i, [VP, VP])
    _sig(lib, "sei_kernel_times_ms", i, [VP, C.POINTER(d), C.POINTER(d), C.POINTER(i)])
    _sig(lib, "sei_kernel_times_by_kind", i, [VP, VP, VP])
    _sig(lib, "sei_visco_setup", i, [VP, d, d, d, d])
    _sig(lib, "sei_num_quantities", i, [VP])
    _sig(lib, "sei_visco_operators", i, [VP, VP, VP, VP, VP, VP])
    _sig(lib, "sei_fit_attenuation", i, [d, d, d, d, C.POINTER(d), C.POINTER(d), VP, VP])
    _sig(lib, "sei_lts_setup", i, [VP, d, i, C.POINTER(i)])
    _sig(lib, "sei_lts_run", i, [VP, i])
    _sig(lib, "sei_lts_clusters", i, [VP, C.POINTER(i), VP, VP])
    _sig(lib, "sei_lts_permutation", i, [VP, VP])
    _sig(lib, "sei_mlp_num_params", i, [])
    _sig(lib, "sei_dr_record_samples", i, [VP, i64])
    _sig(lib, "sei_dr_get_samples", i, [VP, VP, i64, C.POINTER(i64)])
    _sig(lib, "sei_mlp_train", i, [VP, VP, i64, i, C.c_float, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_float)])
    _sig(lib, "sei_mlp_get", i, [VP, VP, VP])
    _sig(lib, "sei_mlp_set", i, [VP, VP, VP])
    _sig(lib, "sei_dr_warm_start", i, [VP, i])
    _sig(lib, "sei_mlp_gradient", i, [VP, VP, VP, i64, VP, C.POINTER(C.c_float)])
    _sig(lib, "sei_mlp_predict", i, [VP, VP, VP, i64, VP])
    _sig(lib, "sei_mlp_gradient_noalloc", i, [VP, VP, VP, i64, VP, C.POINTER(C.c_float)])
    if path is None:
        _lib = lib
    return lib


def nbasis(order):
    return order * (order + 1) * (order + 2) // 6


def padded_basis(order):
    return (nbasis(order) + 3) // 4 * 4


def derivatives_size(order):
    return sum(nbasis(order - i) for i in range(order)) * 9


def _ptr(a):
    return None if a is None else a.ctypes.data_as(VP)


def _colmajor(a, dtype=np.float32):
    return np.ascontiguousarray(np.swapaxes(np.asarray(a), -1, -2), dtype=dtype)


def tc_gemm_check(A, B, terms=3):
    """D = A B^T for one 128 x N x K tile on the tensor cores (diagnostic of the TC conventions)."""
    lib = load_library()
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    D = np.empty((A.shape[0], B.shape[0]), np.float32)
    rc = lib.sei_tc_gemm_check(_ptr(A), _ptr(B), _ptr(D), B.shape[0], A.shape[1], terms)
    if rc != SEI_OK:
        raise SeiError(rc, "sei_tc_gemm_check")
    return D


def device_clock_khz(device=0):
    """Maximum SM clock of a device in kHz (the proxy's cycle count is time x this clock)."""
    lib = load_library()
    k = C.c_int()
    rc = lib.sei_device_clock_khz(int(device), C.byref(k))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_device_clock_khz")
    return k.value


def tc_layout_check(A, B, b_mn=0, lbo_is_k=0, a_mn=0):
    """All 128 TMEM lanes after one M x N x K FP16 tile D = A B^T (A: M x K, B: N x K)."""
    lib = load_library()
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    nc = (B.shape[0] + 15) // 16 * 16
    D = np.empty((128, nc), np.float32)
    rc = lib.sei_tc_layout_check(_ptr(A), _ptr(B), _ptr(D), A.shape[0], B.shape[0], A.shape[1], int(b_mn), int(lbo_is_k),
                                 int(a_mn))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_tc_layout_check")
    return D


def fit_attenuation(mu, lam, qp, qs, freq_central, freq_ratio):
    """(unrelaxed mu, lambda, omega [3], theta [3][3]) of the library's attenuation fit."""
    lib = load_library()
    m, l = C.c_double(mu), C.c_double(lam)
    om, th = np.empty(3), np.empty(9)
    rc = lib.sei_fit_attenuation(qp, qs, freq_central, freq_ratio, C.byref(m), C.byref(l), _ptr(om), _ptr(th))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_fit_attenuation")
    return m.value, l.value, om, th.reshape(3, 3)


def plasticity_relax_factor(tv, dt):
    """1 - exp(-dt / tv), 1 for tv <= 0 (sei_plasticity_relax_factor)."""
    return load_library().sei_plasticity_relax_factor(float(tv), float(dt))


def plasticity_nodes(order):
    """The library's default plasticity nodes [B][3] (equispaced lattice, sei_plasticity_nodes)."""
    out = np.empty((nbasis(order), 3), np.float64)
    rc = load_library().sei_plasticity_nodes(int(order), _ptr(out))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_plasticity_nodes")
    return out


def mlp_num_params():
    return load_library().sei_mlp_num_params()


def mlp_gradient(params, norm, samples):
    """(gradient, loss) of the warm-start network's mean-squared loss over samples [n][6], on the GPU."""
    lib = load_library()
    params = np.ascontiguousarray(params, np.float32)
    norm = np.ascontiguousarray(norm, np.float32)
    samples = np.ascontiguousarray(samples, np.float32)
    g = np.empty(lib.sei_mlp_num_params(), np.float32)
    loss = C.c_float()
    rc = lib.sei_mlp_gradient(_ptr(params), _ptr(norm), _ptr(samples), samples.shape[0], _ptr(g), C.byref(loss))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_mlp_gradient")
    return g, loss.value


def mlp_predict(params, norm, samples):
    """log10 slip rate predicted for each sample [n][6] (last column ignored), on the GPU."""
    lib = load_library()
    params = np.ascontiguousarray(params, np.float32)
    norm = np.ascontiguousarray(norm, np.float32)
    samples = np.ascontiguousarray(samples, np.float32)
    out = np.empty(samples.shape[0], np.float32)
    rc = lib.sei_mlp_predict(_ptr(params), _ptr(norm), _ptr(samples), samples.shape[0], _ptr(out))
    if rc != SEI_OK:
        raise SeiError(rc, "sei_mlp_predict")
    return out


class Context:
    """One device-resident mesh and its element-update kernels (sei_ctx)."""

    def __init__(self, order: int, device: int = 0, precision: int = 0, store_derivatives: bool = False):
        self.lib = load_library()
        self.order = order
        self.B = nbasis(order)
        self.nq = 9
        cfg = _Config(order, device, precision, int(store_derivatives))
        h = VP()
        rc = self.lib.sei_create(C.byref(cfg), C.byref(h))
        if rc != SEI_OK:
            raise SeiError(rc, f"sei_create(order={order}, device={device}, precision={precision}) failed")
        self.h = h
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.sei_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != SEI_OK:
            msg = self.lib.sei_last_error(self.h)
            raise SeiError(rc, f"{what}: {msg.decode() if msg else ''}")

    # -- set-up ------------------------------------------------------------------------
    def build_periodic_cube(self, nx, ny, nz, h=100.0, rho=2700.0, vp=6000.0, vs=3464.0, perturb=0.0, seed=1,
                            fault_plane=-1, grading=1.0, lts_profile=0):
        p = _CubeParams(nx, ny, nz, h, rho, vp, vs, perturb, seed, fault_plane, grading, int(lts_profile))
        n = C.c_int64()
        self._check(self.lib.sei_build_periodic_cube(self.h, C.byref(p), C.byref(n)), "sei_build_periodic_cube")
        self.n = n.value
        return self.n

    def set_mesh(self, geometry, connect, material, boundary=None, boundary_format="i32", identify=None,
                 fault_ref=(0.0, 0.0, 0.0), fault_ref_method="point"):
        """Mesh from the arrays of a PUML file (sei_set_mesh): geometry [nv, 3], connect [n, 4],
        material [n, 3] (rho, mu, lambda), boundary [n] (i32 / i64) or [n, 4] (i32x4), identify [nv]
        (identify-vertex topology).  Returns (cells, fault faces)."""
        geo = np.ascontiguousarray(geometry, np.float64)
        con = np.ascontiguousarray(connect, np.int64)
        mat = np.ascontiguousarray(material, np.float64)
        bnd = None
        if boundary is not None:
            dt = {"i32": np.uint32, "i64": np.uint64, "i32x4": np.int32}[boundary_format]
            bnd = np.ascontiguousarray(boundary, dt)
        idn = np.ascontiguousarray(identify, np.int64) if identify is not None else None
        m = _Mesh(geo.shape[0], geo.ctypes.data, con.shape[0], con.ctypes.data,
                  bnd.ctypes.data if bnd is not None else None, BOUNDARY_FORMATS[boundary_format],
                  idn.ctypes.data if idn is not None else None, mat.ctypes.data,
                  (C.c_double * 3)(*fault_ref), FAULT_REF_METHODS[fault_ref_method])
        n, nf = C.c_int64(), C.c_int64()
        self._check(self.lib.sei_set_mesh(self.h, C.byref(m), C.byref(n), C.byref(nf)), "sei_set_mesh")
        self.n = n.value
        return self.n, nf.value

    # -- output ----------------------------------------------------------------------
    def receivers_setup(self, points, interval, quantities=range(9), rotation=False, strain=False):
        """Receivers at points [n, 3] sampled every `interval` (sei_receivers_setup); returns the
        containing cells.  quantities: indices 0..8 kept in the output."""
        pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        mask = 0
        for q in quantities:
            mask |= 1 << int(q)
        cells = np.empty(len(pts), np.int64)
        derived = (1 if rotation else 0) | (2 if strain else 0)
        self._check(self.lib.sei_receivers_setup(self.h, len(pts), _ptr(pts) if len(pts) else None, float(interval),
                                                 mask, derived, _ptr(cells) if len(pts) else None),
                    "sei_receivers_setup")
        self.nrecv = len(pts)
        return cells

    def receivers_read(self, max_samples=1 << 20):
        """Samples staged so far: array [samples, receivers, columns] (column 0 is the time)."""
        ncols = self.lib.sei_receivers_columns(self.h)
        if ncols == 0:
            return np.zeros((0, 0, 0))
        total = []
        while True:
            chunk = np.empty((1024, self.nrecv, ncols), np.float64)
            got = C.c_int64()
            self._check(self.lib.sei_receivers_read(self.h, _ptr(chunk), 1024, C.byref(got)), "sei_receivers_read")
            total.append(chunk[: got.value])
            if got.value < 1024 or sum(len(t) for t in total) >= max_samples:
                break
        return np.concatenate(total)

    def time(self):
        t = C.c_double()
        self._check(self.lib.sei_get_time(self.h, C.byref(t)), "sei_get_time")
        return t.value

    def set_time(self, t):
        self._check(self.lib.sei_set_time(self.h, float(t)), "sei_set_time")

    def plasticity_setup(self, bulk_friction, plast_co, s0, tv=0.1, nodes=None, per_node=False):
        """Off-fault plasticity (sei_plasticity_setup).  Per cell: bulk_friction [n], plast_co [n],
        s0 [n, 6]; per_node: [n, B], [n, B], [n, B, 6].  nodes [B, 3] (None: the equispaced lattice)."""
        bf = np.ascontiguousarray(bulk_friction, np.float64)
        co = np.ascontiguousarray(plast_co, np.float64)
        s0 = np.ascontiguousarray(s0, np.float64)
        nd = None if nodes is None else np.ascontiguousarray(nodes, np.float64).reshape(-1, 3)
        want = (self.n, self.B) if per_node else (self.n,)
        if bf.shape != want or co.shape != want or s0.shape != want + (6,):
            raise ValueError(f"plasticity parameters must be {want} and {want + (6,)}")
        if nd is not None and nd.shape != (self.B, 3):
            raise ValueError(f"nodes must be [{self.B}, 3]")
        self._check(self.lib.sei_plasticity_setup(self.h, _ptr(nd) if nd is not None else None, float(tv), _ptr(bf),
                                                  _ptr(co), _ptr(s0), int(bool(per_node))), "sei_plasticity_setup")

    def plasticity_disable(self):
        self._check(self.lib.sei_plasticity_disable(self.h), "sei_plasticity_disable")

    def plasticity_strain(self):
        """Nodal plastic strain [n, 7, B]: xx, yy, zz, xy, yz, xz, then eta."""
        out = np.empty((self.n, 7, self.B), np.float32)
        self._check(self.lib.sei_plasticity_get_strain(self.h, _ptr(out)), "sei_plasticity_get_strain")
        return out

    def plasticity_yield_count(self):
        v = C.c_int64()
        self._check(self.lib.sei_plasticity_yield_count(self.h, C.byref(v)), "sei_plasticity_yield_count")
        return v.value

    def fault_output_setup(self, every, fields):
        ids = np.ascontiguousarray([DR_FIELDS[f] if isinstance(f, str) else int(f) for f in fields], np.int32)
        self._check(self.lib.sei_fault_output_setup(self.h, int(every), _ptr(ids) if len(ids) else None, len(ids)),
                    "sei_fault_output_setup")
        self.fault_fields = len(ids)

    def fault_output_read(self):
        """Snapshots so far: (times [k], fields [k, nfields, nfaces, npts])."""
        per = 1 + self.fault_fields * self.nfaces * self.npts
        out = []
        while True:
            chunk = np.empty((16, per), np.float64)
            got = C.c_int64()
            self._check(self.lib.sei_fault_output_read(self.h, _ptr(chunk), 16, C.byref(got)), "sei_fault_output_read")
            out.append(chunk[: got.value])
            if got.value < 16:
                break
        a = np.concatenate(out)
        return a[:, 0], a[:, 1:].reshape(len(a), self.fault_fields, self.nfaces, self.npts)

    def set_cells(self, star, aplus, aminus, neighbor, side, orient, face_type):
        n = star.shape[0]
        arrs = [_colmajor(star), _colmajor(aplus), _colmajor(aminus), np.ascontiguousarray(neighbor, np.int32),
                np.ascontiguousarray(side, np.int8), np.ascontiguousarray(orient, np.int8),
                np.ascontiguousarray(face_type, np.int8)]
        self._check(self.lib.sei_set_cells(self.h, n, *[_ptr(a) for a in arrs]), "sei_set_cells")
        self.n = n

    def get_cells(self):
        n = self.n
        star = np.empty((n, 3, 9, 9), np.float32)
        ap = np.empty((n, 4, 9, 9), np.float32)
        am = np.empty((n, 4, 9, 9), np.float32)
        nb = np.empty((n, 4), np.int32)
        side = np.empty((n, 4), np.int8)
        orient = np.empty((n, 4), np.int8)
        ft = np.empty((n, 4), np.int8)
        self._check(self.lib.sei_get_cells(self.h, *[_ptr(a) for a in (star, ap, am, nb, side, orient, ft)]), "sei_get_cells")
        sw = lambda a: np.swapaxes(a, -1, -2)  # stored column-major -> numpy [q, p]
        return {"star": sw(star), "AplusT": sw(ap), "AminusT": sw(am), "neighbor": nb, "side": side, "orient": orient,
                "face_type": ft}

    def get_geometry(self):
        n = self.n
        v = np.empty((n, 4, 3), np.float64)
        m = np.empty((n, 3), np.float64)
        t = np.empty((n, 4), np.int64)
        self._check(self.lib.sei_get_geometry(self.h, _ptr(v), _ptr(m), _ptr(t)), "sei_get_geometry")
        return v, m, t

    def cfl_timestep(self, cfl=0.5):
        d = C.c_double()
        self._check(self.lib.sei_cfl_timestep(self.h, cfl, C.byref(d)), "sei_cfl_timestep")
        return d.value

    # -- data ---------------------------------------------------------------------------
    def set_dofs(self, dofs):
        a = np.ascontiguousarray(dofs, np.float32)
        assert a.shape == (self.n, self.nq, self.B), a.shape
        self._check(self.lib.sei_set_dofs(self.h, _ptr(a)), "sei_set_dofs")

    def get_dofs(self):
        a = np.empty((self.n, self.nq, self.B), np.float32)
        self._check(self.lib.sei_get_dofs(self.h, _ptr(a)), "sei_get_dofs")
        return a

    def get_time_integrated(self):
        a = np.empty((self.n, self.nq, self.B), np.float32)
        self._check(self.lib.sei_get_time_integrated(self.h, _ptr(a)), "sei_get_time_integrated")
        return a

    def get_derivatives(self):
        a = np.empty((self.n, derivatives_size(self.order)), np.float32)
        self._check(self.lib.sei_get_derivatives(self.h, _ptr(a)), "sei_get_derivatives")
        return a

    # -- kernels ------------------------------------------------------------------------
    def set_option(self, option, value):
        self._check(self.lib.sei_set_option(self.h, option, int(value)), "sei_set_option")

    def get_option(self, option):
        v = C.c_int()
        self._check(self.lib.sei_get_option(self.h, option, C.byref(v)), "sei_get_option")
        return v.value

    def compute_ader(self, dt, coeffs=None):
        """Spacetime::computeAder: I = sum_i coeffs[i] dQ_i (coeffs default: integrate(0, dt))."""
        cp = None
        if coeffs is not None:
            cp = np.ascontiguousarray(coeffs, np.float64)
            if cp.shape != (self.order,):
                raise ValueError(f"coeffs must have {self.order} entries")
        self._check(self.lib.sei_compute_ader(self.h, _ptr(cp), dt), "sei_compute_ader")

    def compute_local_integral(self):
        self._check(self.lib.sei_compute_local_integral(self.h), "sei_compute_local_integral")

    def compute_ader_local(self, dt):
        self._check(self.lib.sei_compute_ader_local(self.h, dt), "sei_compute_ader_local")

    def compute_neighbors_integral(self):
        self._check(self.lib.sei_compute_neighbors_integral(self.h), "sei_compute_neighbors_integral")

    def run(self, kernel, dt, nsteps):
        k = KERNELS[kernel] if isinstance(kernel, str) else kernel
        self._check(self.lib.sei_run(self.h, k, dt, nsteps), f"sei_run({kernel})")

    def run_host(self, kernel, dt, nsteps, dofs_in, dofs_out):
        k = KERNELS[kernel] if isinstance(kernel, str) else kernel
        self._check(self.lib.sei_run_host(self.h, k, dt, nsteps, _ptr(dofs_in), _ptr(dofs_out)), f"sei_run_host({kernel})")

    def sync(self):
        self._check(self.lib.sei_sync(self.h), "sei_sync")

    # -- dynamic rupture ------------------------------------------------------------------
    def dr_setup(self, params: "RSParams"):
        nf = C.c_int64()
        self._check(self.lib.sei_dr_setup(self.h, C.byref(params), C.byref(nf)), "sei_dr_setup")
        self.nfaces = nf.value
        self.npts = self.lib.sei_dr_num_points(self.order)
        return self.nfaces

    def dr_setup_rate_state(self, params: "RSParams", law: int):
        """Rate-and-state fault with law 0 (fast velocity weakening), 4 (aging), 5 (slip) or 6 (severe)."""
        nf = C.c_int64()
        self._check(self.lib.sei_dr_setup_rate_state(self.h, C.byref(params), int(law), C.byref(nf)),
                    "sei_dr_setup_rate_state")
        self.nfaces = nf.value
        self.npts = self.lib.sei_dr_num_points(self.order)
        return self.nfaces

    def dr_setup_imposed(self, params: "ISRParams"):
        nf = C.c_int64()
        self._check(self.lib.sei_dr_setup_imposed(self.h, C.byref(params), C.byref(nf)), "sei_dr_setup_imposed")
        self.nfaces = nf.value
        self.npts = self.lib.sei_dr_num_points(self.order)
        return self.nfaces

    def dr_set_thermal_pressurization(self, on=True, params: "TPParams" = None):
        self._check(self.lib.sei_dr_set_thermal_pressurization(self.h, int(on), C.byref(params) if params else None),
                    "sei_dr_set_thermal_pressurization")

    def dr_setup_lsw(self, params: "LSWParams"):
        nf = C.c_int64()
        self._check(self.lib.sei_dr_setup_lsw(self.h, C.byref(params), C.byref(nf)), "sei_dr_setup_lsw")
        self.nfaces = nf.value
        self.npts = self.lib.sei_dr_num_points(self.order)
        return self.nfaces

    def dr_law(self):
        return self.lib.sei_dr_law(self.h)

    def dr_set_nucleation(self, on=True, t0=0.0, s0=0.0):
        self._check(self.lib.sei_dr_set_nucleation(self.h, int(on), t0, s0), "sei_dr_set_nucleation")

    def dr_time(self):
        t = C.c_double()
        self._check(self.lib.sei_dr_get_time(self.h, C.byref(t)), "sei_dr_get_time")
        return t.value

    def dr_set_time(self, t):
        self._check(self.lib.sei_dr_set_time(self.h, float(t)), "sei_dr_set_time")

    def dr_faces(self):
        nf = self.lib.sei_dr_num_faces(self.h)
        cells = np.empty((nf, 2), np.int32)
        sides = np.empty((nf, 3), np.int8)
        tinvt = np.empty((nf, 9, 9), np.float32)
        fsp = np.empty((nf, 9, 9), np.float32)
        fsm = np.empty((nf, 9, 9), np.float32)
        imp = np.empty((nf, 8), np.float64)
        self._check(self.lib.sei_dr_get_faces(self.h, *[_ptr(a) for a in (cells, sides, tinvt, fsp, fsm, imp)]),
                    "sei_dr_get_faces")
        sw = lambda a: np.swapaxes(a, -1, -2)
        return {"cells": cells, "sides": sides, "TinvT": sw(tinvt), "fluxSolverPlus": sw(fsp),
                "fluxSolverMinus": sw(fsm), "imp": imp}

    def dr_state(self, field):
        out = np.empty((self.nfaces, self.npts), np.float64)
        self._check(self.lib.sei_dr_get_state(self.h, DR_FIELDS[field], _ptr(out)), "sei_dr_get_state")
        return out

    def dr_set_state(self, field, values):
        a = np.ascontiguousarray(values, np.float64)
        assert a.shape == (self.nfaces, self.npts)
        self._check(self.lib.sei_dr_set_state(self.h, DR_FIELDS[field], _ptr(a)), "sei_dr_set_state")

    def dr_imposed(self):
        p = np.empty((self.nfaces, 9, self.npts), np.float32)
        m = np.empty((self.nfaces, 9, self.npts), np.float32)
        self._check(self.lib.sei_dr_get_imposed(self.h, _ptr(p), _ptr(m)), "sei_dr_get_imposed")
        return p, m

    def dr_newton_iterations(self, first=False):
        """(total iterations, points); with first=True also the iterations of the first solves."""
        t, n, f = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.sei_dr_newton_iterations(self.h, C.byref(t), C.byref(n), C.byref(f)),
                    "sei_dr_newton_iterations")
        return (t.value, n.value, f.value) if first else (t.value, n.value)

    def dr_newton_iterations32(self):
        """Float32 pre-iterations of all solves (SEI_OPT_DR_REFINE32) since the last reset."""
        t = C.c_int64()
        self._check(self.lib.sei_dr_newton_iterations32(self.h, C.byref(t)), "sei_dr_newton_iterations32")
        return t.value

    def dr_reset_counters(self):
        self._check(self.lib.sei_dr_reset_counters(self.h), "sei_dr_reset_counters")

    def dr_faces_step(self, dt):
        self._check(self.lib.sei_dr_faces_step(self.h, dt), "sei_dr_faces_step")

    def dr_slots(self):
        out = np.empty(self.n, np.int32)
        self._check(self.lib.sei_dr_get_slots(self.h, _ptr(out)), "sei_dr_get_slots")
        return out

    def get_derivatives_slots(self, nslots):
        a = np.empty((nslots, derivatives_size(self.order)), np.float32)
        self._check(self.lib.sei_get_derivatives(self.h, _ptr(a)), "sei_get_derivatives")
        return a

    def dr_record_samples(self, capacity):
        self._check(self.lib.sei_dr_record_samples(self.h, int(capacity)), "sei_dr_record_samples")

    def dr_samples(self):
        cnt = C.c_int64()
        self._check(self.lib.sei_dr_get_samples(self.h, None, 0, C.byref(cnt)), "sei_dr_get_samples")
        out = np.empty((cnt.value, 6), np.float32)
        self._check(self.lib.sei_dr_get_samples(self.h, _ptr(out), cnt.value, C.byref(cnt)), "sei_dr_get_samples")
        return out

    def mlp_train(self, samples=None, steps=2000, lr=3e-3, seed=1):
        """Trains the warm-start network on the GPU; returns (first loss, last loss)."""
        s = None if samples is None else np.ascontiguousarray(samples, np.float32)
        a, b = C.c_float(), C.c_float()
        self._check(self.lib.sei_mlp_train(self.h, _ptr(s), 0 if s is None else s.shape[0], steps, lr, seed, C.byref(a),
                                           C.byref(b)), "sei_mlp_train")
        return a.value, b.value

    def mlp_get(self):
        p = np.empty(self.lib.sei_mlp_num_params(), np.float32)
        nrm = np.empty(16, np.float32)
        self._check(self.lib.sei_mlp_get(self.h, _ptr(p), _ptr(nrm)), "sei_mlp_get")
        return p, nrm

    def mlp_set(self, params, norm):
        p = np.ascontiguousarray(params, np.float32)
        nrm = np.ascontiguousarray(norm, np.float32)
        self._check(self.lib.sei_mlp_set(self.h, _ptr(p), _ptr(nrm)), "sei_mlp_set")

    def dr_warm_start(self, on=True):
        self._check(self.lib.sei_dr_warm_start(self.h, int(on)), "sei_dr_warm_start")

    def visco_setup(self, qp=100.0, qs=50.0, freq_central=0.5, freq_ratio=100.0):
        """Viscoelastic equations, 3 mechanisms: the DOFs become [n][27][B]."""
        self._check(self.lib.sei_visco_setup(self.h, qp, qs, freq_central, freq_ratio), "sei_visco_setup")
        self.nq = self.lib.sei_num_quantities(self.h)

    def visco_operators(self):
        """grad [n][3][3], theta [n][3][3], W+ and W- [n][4][9][6], omega [3]."""
        n = self.n
        g, t = np.empty((n, 3, 3), np.float32), np.empty((n, 3, 3), np.float32)
        wp, wm = np.empty((n, 4, 6, 9), np.float32), np.empty((n, 4, 6, 9), np.float32)
        om = np.empty(3, np.float64)
        self._check(self.lib.sei_visco_operators(self.h, _ptr(g), _ptr(t), _ptr(wp), _ptr(wm), _ptr(om)),
                    "sei_visco_operators")
        return g, t, np.swapaxes(wp, -1, -2), np.swapaxes(wm, -1, -2), om

    def lts_setup(self, cfl=0.5, max_clusters=8):
        """Rate-2 local time stepping; reorders the cells by cluster.  Returns the cluster count."""
        k = C.c_int()
        self._check(self.lib.sei_lts_setup(self.h, cfl, max_clusters, C.byref(k)), "sei_lts_setup")
        return k.value

    def lts_run(self, ncycles=1):
        self._check(self.lib.sei_lts_run(self.h, ncycles), "sei_lts_run")

    def lts_clusters(self):
        """(start [ncl + 1], dt [ncl]) of the clusters."""
        k = C.c_int()
        self._check(self.lib.sei_lts_clusters(self.h, C.byref(k), None, None), "sei_lts_clusters")
        start = np.zeros(k.value + 1, np.int64)
        dt = np.zeros(k.value, np.float64)
        self._check(self.lib.sei_lts_clusters(self.h, C.byref(k), _ptr(start), _ptr(dt)), "sei_lts_clusters")
        return start, dt

    def lts_permutation(self):
        out = np.zeros(self.n, np.int64)
        self._check(self.lib.sei_lts_permutation(self.h, _ptr(out)), "sei_lts_permutation")
        return out

    def set_profiling(self, on=True):
        self._check(self.lib.sei_set_profiling(self.h, int(on)), "sei_set_profiling")

    def kernel_times_ms(self):
        """(local ms, neighbour ms, launches) summed over the last run with profiling on."""
        a, b, n = C.c_double(), C.c_double(), C.c_int()
        self._check(self.lib.sei_kernel_times_ms(self.h, C.byref(a), C.byref(b), C.byref(n)), "sei_kernel_times_ms")
        return a.value, b.value, n.value

    def kernel_times_by_kind(self):
        """{kind: (ms, launches)} of the last run with profiling on: ader, neighbor, fault, lint."""
        ms = np.zeros(4, np.float64)
        cnt = np.zeros(4, np.int32)
        self._check(self.lib.sei_kernel_times_by_kind(self.h, _ptr(ms), _ptr(cnt)), "sei_kernel_times_by_kind")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(("ader", "neighbor", "fault", "lint"))}

    def metrics(self, kernel):
        """Per-cell estimate of one step of a proxy kernel (sei_metrics): non-zero flops, hardware
        flops and compulsory bytes."""
        out = _Perf()
        self._check(self.lib.sei_metrics(self.h, KERNELS[kernel], C.byref(out)), "sei_metrics")
        return {"nonzero_flop": out.nonzero_flop, "hardware_flop": out.hardware_flop, "bytes": out.bytes}

    def last_run_ms(self):
        d = C.c_double()
        self._check(self.lib.sei_last_run_ms(self.h, C.byref(d)), "sei_last_run_ms")
        return d.value

    def autotune(self, dt, steps=5):
        """Times every variant of the step on this mesh, keeps the fastest (sei_autotune)."""
        r = _Tune()
        self._check(self.lib.sei_autotune(self.h, dt, int(steps), C.byref(r)), "sei_autotune")
        return {k: getattr(r, k) for k, _ in _Tune._fields_}
