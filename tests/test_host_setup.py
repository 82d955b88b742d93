"""Host side of the product (C++, through the C ABI on a host-only context) vs the oracle.

The C++ set-up builds the mesh, face relations, star matrices and flux solvers
(src/Initializer/Model/CellLocalMatrices.cpp:66-296); the oracle recomputes the relations
and operators from the same geometry and materials in float64.  No GPU is needed.
"""
import re
import os

import numpy as np
import pytest

from tests.helpers import oracle_inputs_from_geometry


def _ctx(order=4):
    from seissol_gb300 import Context
    return Context(order, device=-1)


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "sei_gb300.h")).read()
    names = set(re.findall(r"^\s*(?:int|int64_t|void|const char\*)\s+(sei_\w+)\(", hdr, re.M))
    assert len(names) >= 20
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sei_version() == 1


@pytest.mark.parametrize("perturb", [0.0, 0.1])
def test_operators_match_oracle(built_lib, perturb):
    with _ctx(4) as ctx:
        n = ctx.build_periodic_cube(4, 4, 4, perturb=perturb, seed=11)
        assert n == 320
        coords, material, topo = ctx.get_geometry()
        cells = ctx.get_cells()
    # positively oriented tetrahedra
    e = coords[:, 1:] - coords[:, :1]
    assert (np.linalg.det(e) > 0).all()
    nb, side, orient, ops = oracle_inputs_from_geometry(coords, material, topo)
    assert np.array_equal(cells["neighbor"], nb)
    assert np.array_equal(cells["side"], side)
    assert np.array_equal(cells["orient"], orient)
    assert (cells["face_type"] == 0).all()
    for key in ("star", "AplusT", "AminusT"):
        a, b = cells[key].astype(np.float64), ops[key]
        scale = np.abs(b).max(axis=(-1, -2), keepdims=True)
        assert np.abs(a - b).max() <= 1e-6 * scale.max(), key
        assert (np.abs(a - b) <= 2e-6 * scale + 1e-30).all(), key


def test_material_perturbation_range(built_lib):
    with _ctx(4) as ctx:
        ctx.build_periodic_cube(4, 4, 4, perturb=0.1, seed=3)
        _, material, _ = ctx.get_geometry()
    rho, mu, lam = material.T
    vs = np.sqrt(mu / rho)
    vp = np.sqrt((lam + 2 * mu) / rho)
    assert (rho >= 2700 * 0.9 - 1e-9).all() and (rho <= 2700 * 1.1 + 1e-9).all()
    assert (vs >= 3464 * 0.9 - 1e-6).all() and (vs <= 3464 * 1.1 + 1e-6).all()
    assert (vp >= 6000 * 0.9 - 1e-6).all() and (vp <= 6000 * 1.1 + 1e-6).all()
    assert np.std(rho) > 10


def test_cfl_timestep_matches_oracle(built_lib):
    from oracle import dg_setup
    with _ctx(6) as ctx:
        ctx.build_periodic_cube(4, 4, 4, perturb=0.1, seed=5)
        dt = ctx.cfl_timestep(0.5)
        coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    assert dt == pytest.approx(dg_setup.cfl_timestep(coords, vp, 6, 0.5).min(), rel=1e-12)


def test_invalid_arguments_are_errors(built_lib):
    from seissol_gb300 import SeiError
    with _ctx(4) as ctx:
        with pytest.raises(SeiError, match="SEI_ERR_ARG"):
            ctx.build_periodic_cube(3, 4, 4)
        with pytest.raises(SeiError, match="SEI_ERR_ARG"):
            ctx.build_periodic_cube(4, 4, 4, rho=-1.0)
        with pytest.raises(SeiError, match="SEI_ERR_STATE"):
            ctx.get_dofs()  # host-only context holds no device data
    with pytest.raises(SeiError, match="SEI_ERR_UNSUPPORTED"):
        from seissol_gb300 import Context
        Context(3, device=-1)


def test_metrics_per_kernel(built_lib):
    """sei_metrics: non-zero flops of the generated kernels and compulsory bytes per cell and step
    (order 6: 10,964 B for kernel all, the step model of the elastic configuration)."""
    import ctypes as C
    from seissol_gb300 import Context, KERNELS
    from seissol_gb300.lib import _Perf
    from seissol_gb300.codegen.gen_kernels import nnz_flops
    f = nnz_flops(6)
    with Context(6, device=-1) as ctx:
        out = {}
        for name in ("all", "local", "ader", "localwoader", "neigh"):
            p = _Perf()
            assert ctx.lib.sei_metrics(ctx.h, KERNELS[name], C.byref(p)) == 0
            out[name] = (p.nonzero_flop, p.hardware_flop, p.bytes)
        p = _Perf()
        assert ctx.lib.sei_metrics(ctx.h, KERNELS["all_dr"], C.byref(p)) != 0
    assert out["all"][0] == pytest.approx(f["ader"] + f["local"] + f["neighbor"])
    assert out["local"][0] == pytest.approx(f["ader"] + f["local"])
    assert out["neigh"][0] == pytest.approx(f["neighbor"])
    assert out["all"][2] == 10964
    assert out["ader"][2] == 2 * 2016 + 288
