"""GPU viscoelastic element update (27 quantities, 3 mechanisms) through the C ABI against the dense
FP64 oracle (oracle/visco.py), whose operators are rebuilt independently from the context's
geometry and relaxed material (Qp 100, Qs 50, central frequency 0.5 Hz, ratio 100).

Tolerances (per quantity, FP32 GPU vs FP64 oracle on the same inputs): one ADER 2e-5 relative L2;
one local integral and one neighbour flux: the error of the update within 2e-5 of the update plus
1e-6 of the field (the FP32 storage of Q: the memory variables of the slowest mechanism change by
~1e-4 of their value in one application); ten steps of kernel 'all' 1e-4 relative L2.
"""
import numpy as np
import pytest

from oracle import visco
from tests.helpers import rel_l2_per_quantity


def _update_errors(q_new, q_old, ref):
    """Per quantity: |q_new - ref| / (|ref - q_old| + 0.05 |q_old|), compared with 2e-5 below, i.e.
    an update error within 2e-5 of the update plus 1e-6 of the field."""
    out = []
    for k in range(q_new.shape[1]):
        num = np.linalg.norm(q_new[:, k].astype(np.float64) - ref[:, k])
        den = np.linalg.norm(ref[:, k] - q_old[:, k]) + 0.05 * np.linalg.norm(q_old[:, k])
        out.append(num / den)
    return out

pytestmark = pytest.mark.gpu

QP, QS, FC, RATIO = 100.0, 50.0, 0.5, 100.0


def _setup(order, dims=(4, 4, 4), seed=8):
    from seissol_gb300 import Context
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(*dims, perturb=0.1, seed=seed)
    ctx.visco_setup(QP, QS, FC, RATIO)
    assert ctx.nq == 27
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    mats, thetas = [], []
    for rho, mu, lam in material:
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, QP, QS, FC, RATIO)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    ops = visco.cell_operators(coords, np.array(mats), omega, np.array(thetas), cells["neighbor"])
    rng = np.random.default_rng(seed)
    q0 = rng.uniform(-1, 1, (n, 27, ctx.B)).astype(np.float32)
    ctx.set_dofs(q0)
    return ctx, n, cells, ops, q0


@pytest.mark.parametrize("order", [4, 5])
def test_visco_kernels_one_application(built_lib, order):
    ctx, n, cells, ops, q0 = _setup(order)
    o = visco.Visco(order)
    dt = ctx.cfl_timestep(0.5)
    ctx.compute_ader(dt)
    ctx.sync()
    i_gpu = ctx.get_time_integrated()
    i_ref = o.ader(q0.astype(np.float64), ops["star"], ops["ET"], dt)
    errs = rel_l2_per_quantity(i_gpu, i_ref)
    assert max(errs) < 2e-5, errs
    ctx.compute_local_integral()
    ctx.sync()
    q_loc = ctx.get_dofs()
    ref = o.local(q0.astype(np.float64), i_gpu.astype(np.float64), ops["star"], ops["ET"], ops["AplusT"],
                  cells["face_type"])
    errs = _update_errors(q_loc, q0, ref)
    assert max(errs) < 2e-5, errs
    ctx.compute_neighbors_integral()
    ctx.sync()
    ref_n = o.neighbor(q_loc.astype(np.float64), i_gpu.astype(np.float64), ops["AminusT"], cells["neighbor"],
                       cells["side"], cells["orient"], cells["face_type"])
    errs = _update_errors(ctx.get_dofs(), q_loc, ref_n)
    assert max(errs) < 2e-5, errs
    ctx.close()


@pytest.mark.parametrize("order", [4, 5])
def test_visco_ten_steps(built_lib, order):
    ctx, n, cells, ops, q0 = _setup(order, seed=9)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 10)
    ctx.sync()
    ref = visco.Visco(order).steps(q0.astype(np.float64), ops, cells["neighbor"], cells["side"], cells["orient"],
                                   cells["face_type"], dt, 10)
    errs = rel_l2_per_quantity(ctx.get_dofs(), ref)
    assert max(errs) < 1e-4, errs
    ctx.close()


def test_visco_rejects_unbuilt(built_lib):
    from seissol_gb300 import Context, SeiError
    ctx = Context(6, device=0)
    ctx.build_periodic_cube(4, 4, 4)
    with pytest.raises(SeiError, match="SEI_ERR_UNSUPPORTED"):
        ctx.visco_setup()
    ctx.close()
    ctx, *_ = _setup(4)
    with pytest.raises(SeiError, match="SEI_ERR_UNSUPPORTED"):
        ctx.run("all_dr", 1e-4, 1)
    with pytest.raises(SeiError):
        ctx.lts_setup(0.5, 4)
    ctx.close()
