"""Off-fault plasticity on the GPU (sei_plasticity_setup) against the float64 restatement
oracle/plasticity.py driven by the oracle's element update.

Workloads: periodic cubes of 4 x 4 x 4 cubes (320 tets, material +-10 %), seeded DOFs U[-1, 1],
bulk friction 0.6, cohesion (per cell or per node) such that c cos(phi) is U[0.7, 1.5] times the
median largest nodal tau after one step, initial stress U[-1, 1] MPa, T_v = 0.05 s: a part of the
cells yields in each step; the reference's nodes (fixture) or the default lattice.  Local time
stepping: the graded 640-tet LTS profile, set up before and after the plasticity (its parameters
and strain move with the cells).
Tolerances: DOFs 2e-5 relative L2 per quantity (FP32 and mixed paths); plastic strain and eta
1e-4 relative L2; yielding cell count within 2 % (a node at the threshold may decide differently
in float32; its update is then near zero).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle_py
from oracle import plasticity as P
from tests.helpers import rel_l2, seeded_dofs

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
PIN = json.load(open(os.path.join(HERE, "golden", "plasticity_nb_pin.json")))


# median over cells of the largest nodal tau after one step of the seeded DOFs (Pa)
TAU = {4: 3.8e7, 5: 5.7e7, 6: 8.7e7}


def _params(n, B, per_node, seed, order):
    rng = np.random.default_rng(seed)
    shape = (n, B) if per_node else (n,)
    bf = np.full(shape, 0.6)
    co = rng.uniform(0.7, 1.5, shape) * TAU[order] / np.cos(np.arctan(0.6))
    s0 = rng.uniform(-1e6, 1e6, shape + (6,))
    return bf, co, s0


def _oracle_state(ctx, nodes, bf, co, s0, per_node):
    _, material, _ = ctx.get_geometry()
    v, vinv = P.matrices(ctx.order, nodes)
    s0n, ccos, ssin = P.cell_parameters(bf, co, s0, ctx.B, per_node)
    return v, vinv, s0n, ccos, ssin, material[:, 1]


def _compare(ctx, q_ref, ps_ref, yields_ref):
    q = ctx.get_dofs()
    errs = [rel_l2(q[:, k], q_ref[:, k]) for k in range(9)]
    assert max(errs) < 2e-5, errs
    ps = ctx.plasticity_strain()
    assert ps_ref.any()
    assert rel_l2(ps[:, :6], ps_ref[:, :6]) < 1e-4
    assert rel_l2(ps[:, 6], ps_ref[:, 6]) < 1e-4
    got = ctx.plasticity_yield_count()
    assert abs(got - yields_ref) <= max(2, 0.02 * yields_ref), (got, yields_ref)


@pytest.mark.parametrize("order,precision,per_node,ref_nodes",
                         [(4, 0, False, True), (5, 0, True, True), (6, 0, False, False), (6, 1, True, True)])
def test_steps_with_plasticity_match_oracle(built_lib, order, precision, per_node, ref_nodes):
    from seissol_gb300 import Context
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.1, seed=5)
    B = ctx.B
    nodes = np.array(PIN[str(order)]["nodes"]) if ref_nodes else P.lattice_nodes(order)
    bf, co, s0 = _params(n, B, per_node, order, order)
    ctx.plasticity_setup(bf, co, s0, tv=0.05, nodes=nodes if ref_nodes else None, per_node=per_node)
    v, vinv, s0n, ccos, ssin, mu = _oracle_state(ctx, nodes, bf, co, s0, per_node)
    q = seeded_dofs(n, order, 13).astype(np.float64)
    ctx.set_dofs(q.astype(np.float32))
    dt = ctx.cfl_timestep(0.5)
    cells = ctx.get_cells()
    o = oracle_py.Oracle(order)
    ps = np.zeros((n, 7, B))
    yields = 0
    for _ in range(3):
        q = o.steps(q, cells["star"], cells["AplusT"], cells["AminusT"], cells["neighbor"], cells["side"],
                    cells["orient"], dt, 1, cells["face_type"])
        yields += int(P.apply(q, ps, v, vinv, s0n, ccos, ssin, mu, dt, 0.05).sum())
    assert 0 < yields < 3 * n
    ctx.run("all", dt, 3)
    ctx.sync()
    _compare(ctx, q, ps, yields)
    ctx.close()


@pytest.mark.parametrize("before", [True, False])
def test_lts_with_plasticity_matches_oracle(built_lib, before):
    """One LTS cycle; the plasticity set up before sei_lts_setup (its parameters and strain follow
    the new cell order) or after it."""
    from seissol_gb300 import Context
    order = 4
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(4, 4, 8, h=50.0, perturb=0.1, seed=2024, grading=8.0, lts_profile=1)
    B = ctx.B
    bf, co, s0 = _params(n, B, False, 9, order)
    if before:
        ctx.plasticity_setup(bf, co, s0, tv=0.05)
    ncl = ctx.lts_setup(0.5, 4)
    assert ncl >= 2
    perm = ctx.lts_permutation()
    if before:
        bf, co, s0 = bf[perm], co[perm], s0[perm]
    else:
        ctx.plasticity_setup(bf, co, s0, tv=0.05)
    start, dts = ctx.lts_clusters()
    cl = np.repeat(np.arange(ncl), np.diff(start))
    v, vinv, s0n, ccos, ssin, mu = _oracle_state(ctx, P.lattice_nodes(order), bf, co, s0, False)
    q0 = seeded_dofs(n, order, 17)
    ctx.set_dofs(q0)
    ps = np.zeros((n, 7, B))
    count = [0]

    def hook(idx, dt, Q):
        sub, sps = Q[idx], ps[idx]
        count[0] += int(P.apply(sub, sps, v, vinv, s0n[idx], ccos[idx], ssin[idx], mu[idx], dt, 0.05).sum())
        Q[idx] = sub
        ps[idx] = sps

    q_ref = oracle_py.lts_cycles(oracle_py.Oracle(order), q0, ctx.get_cells(), cl, dts[0], 1, on_correct=hook)
    assert count[0] > 0
    ctx.lts_run(1)
    ctx.sync()
    _compare(ctx, q_ref, ps, count[0])
    ctx.close()


def test_plasticity_errors(built_lib):
    from seissol_gb300 import Context, SeiError
    ctx = Context(4, device=0)
    n = ctx.build_periodic_cube(4, 4, 4)
    bf, co, s0 = _params(n, ctx.B, False, 1, 4)
    with pytest.raises(SeiError):
        ctx.plasticity_strain()  # not set up
    with pytest.raises(SeiError):
        ctx.plasticity_setup(bf, co, s0, tv=0.0)
    bad = np.zeros((ctx.B, 3))  # every node at one point: not unisolvent
    with pytest.raises(SeiError):
        ctx.plasticity_setup(bf, co, s0, nodes=bad)
    ctx.plasticity_setup(bf, co, s0)
    with pytest.raises(SeiError):
        ctx.visco_setup()  # plasticity with the viscoelastic equations is refused
    ctx.plasticity_disable()
    with pytest.raises(SeiError):
        ctx.plasticity_yield_count()
    ctx.close()
