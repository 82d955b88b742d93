"""GPU steps on meshes ingested through sei_set_mesh (PUML arrays) against the FP64 oracle.

Workloads: a bounded 4 x 4 x 4 box of 100 m cubes (320 tets, material +-10 % per cell) with a
free-surface top and outflow sides; with two crossing fault planes x = 2 h (tag 3) and y = 2 h
(tag 65), so that cells along the crossing line carry two fault faces; and an 8 x 4 x 4 box whose
cells grow fourfold along x (640 tets, four rate-2 clusters) for local time stepping.
Tolerances: DOFs 2e-5 relative L2 per quantity after 5 steps (FP32 and mixed paths); fault steps
along the oracle's trajectory as tests/test_gpu_lsw.py; one LTS cycle 1e-4 relative L2.
"""
import numpy as np
import pytest

from oracle import cube_mesh, dg_setup, oracle_py
from tests.helpers import rel_l2, seeded_dofs
from tests import test_gpu_lsw as L

pytestmark = pytest.mark.gpu


def _material(n, seed=3):
    rng = np.random.default_rng(seed)
    rho = 2700.0 * rng.uniform(0.9, 1.1, n)
    vs = 3464.0 * rng.uniform(0.9, 1.1, n)
    vp = 6000.0 * rng.uniform(0.9, 1.1, n)
    mu = rho * vs * vs
    return np.stack([rho, mu, rho * vp * vp - 2 * mu], axis=1)


def _box(order, precision=0, faults=False, graded=False):
    from seissol_gb300 import Context
    nx = 8 if graded else 4
    geo, con, bnd = cube_mesh.box_mesh(nx, 4, 4, fault_x=2 if faults else None, fault_y=2 if faults else None)
    if graded:
        # cells grow along x from 1 to 4 h in every direction: x = h (i + 3 i^2 / (2 nx)), y and z
        # scaled by 1 + 3 i / nx (an orientation-preserving map: every tet stays positive)
        i = geo[:, 0] / 100.0
        s = 1.0 + 3.0 * i / nx
        geo = np.stack([100.0 * (i + 3.0 * i * i / (2 * nx)), geo[:, 1] * s, geo[:, 2] * s], axis=1)
    ctx = Context(order, device=0, precision=precision)
    n, nf = ctx.set_mesh(geo, con, _material(len(con)), boundary=bnd, fault_ref=(-1e4, -1e4, 0.0))
    return ctx, n, nf


@pytest.mark.parametrize("order,precision", [(4, 0), (5, 0), (6, 0), (6, 1)])
def test_bounded_mesh_steps_match_oracle(built_lib, order, precision):
    ctx, n, nf = _box(order, precision)
    assert nf == 0
    cells = ctx.get_cells()
    assert (cells["face_type"] == 2).any() and (cells["neighbor"] < 0).any()
    q0 = seeded_dofs(n, order, 7)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 5)
    ctx.sync()
    o = oracle_py.Oracle(order)
    q_ref = o.steps(q0, cells["star"], cells["AplusT"], cells["AminusT"], cells["neighbor"], cells["side"],
                    cells["orient"], dt, 5, cells["face_type"])
    q = ctx.get_dofs()
    errs = [rel_l2(q[:, k], q_ref[:, k]) for k in range(9)]
    assert max(errs) < 2e-5, errs
    ctx.close()


@pytest.mark.parametrize("order,precision", [(4, 0), (6, 1)])
def test_crossing_faults_lsw_along_oracle(built_lib, order, precision):
    """Slip weakening with forced rupture on a third of the fault faces; cells with two fault faces
    receive both nodal fluxes."""
    from seissol_gb300 import LSWParams
    ctx, n, nf = _box(order, precision, faults=True)
    faces = ctx.dr_faces()
    counts = np.bincount(faces["cells"].reshape(-1), minlength=n)
    assert counts.max() == 2
    p = LSWParams.fault_config(law=1, seed=4, t0=0.0)
    ctx.dr_setup_lsw(p)
    npts = (order + 1) ** 2
    tf = np.full((nf, npts), 1e300)
    tf[: nf // 3] = 0.0
    ctx.dr_set_state("forced_rupture_time", tf)
    q = seeded_dofs(n, order, 9)
    ctx.set_dofs(q)
    state = {k: ctx.dr_state(v) for k, v in L.FIELDS.items()}
    aux = {k: ctx.dr_state(v) for k, v in L.AUX_FIELDS.items()}
    aux.update(time=0.0, t0=p.t0, s0=0.0, nucleate=0, nuc=None, law=1, healing=-1.0, v_star=p.v_star,
               prakash_length=p.prakash_length, tp_exponent=p.tp_proxy_exponent)
    init = L._init(ctx)
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    o = oracle_py.Oracle(order)
    dro = oracle_py.DROracle(order, faces, {})
    a = np.zeros_like(state["v1"])
    for _ in range(6):
        L._push(ctx, q, state, init, aux)
        q, *_ = oracle_py.dr_full_step(o, dro, q, cells, faces, state, a, init, dt, aux=aux)
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        L._compare(ctx, q, state, init, aux, 1)
    assert (np.hypot(state["v1"], state["v2"]) > 1e-3).any()
    ctx.close()


def test_graded_bounded_mesh_lts_matches_oracle(built_lib):
    order = 4
    ctx, n, _ = _box(order, graded=True)
    ncl = ctx.lts_setup(0.5, 4)
    assert ncl >= 2
    cells = ctx.get_cells()
    coords, material, _ = ctx.get_geometry()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 4)
    start, _ = ctx.lts_clusters()
    assert np.array_equal(cl, np.repeat(np.arange(ncl), np.diff(start)))
    q0 = seeded_dofs(n, order, 11)
    ctx.set_dofs(q0)
    ctx.lts_run(1)
    ctx.sync()
    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, cells, cl, dt0, 1)
    q = ctx.get_dofs()
    errs = [rel_l2(q[:, k], q_ref[:, k]) for k in range(9)]
    assert max(errs) < 1e-4, errs
    ctx.close()
