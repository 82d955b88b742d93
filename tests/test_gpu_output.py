"""Output path on the GPU: receivers and fault snapshots against the FP64 restatement.

Receivers (src/Kernels/Receiver.cpp:118-302): periodic cube 4 x 4 x 4 (320 tets, material
+-5 %), 14 points (two sharing a cell), 3 samples per step.  For each step the oracle takes the
GPU's DOFs at the step start (so each step is compared alone): CK derivatives in float64, the
Taylor expansion at the sampling times, projection onto the basis at the point.  Cells and
sampling times exact; values, rotation and strain within 2e-5 of each column's largest magnitude.
Staging: 2,400 samples of 3 receivers (40 per step, several flushes of the device ring, a read
in the middle) come out complete and in order.  Fault snapshots equal the fault state read
directly after the same steps.
"""
import numpy as np
import pytest

from oracle import dg_setup, oracle_py, receivers
from tests.helpers import seeded_dofs

pytestmark = pytest.mark.gpu


def _cube(order, precision=0, fault_plane=-1):
    from seissol_gb300 import Context
    ctx = Context(order, device=0, precision=precision)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.05, seed=2, fault_plane=fault_plane)
    return ctx, n


def _times(t0, interval, dt, steps):
    """Sampling times by repeated addition, grouped per step (ReceiverCluster::calcReceivers)."""
    out, nxt, T = [], t0, t0
    for _ in range(steps):
        cur = []
        while nxt < T + dt:
            cur.append(nxt)
            nxt += interval
        out.append(cur)
        T += dt
    return out


@pytest.mark.parametrize("order,precision", [(4, 0), (5, 0), (6, 0), (6, 1)])
def test_receivers_match_oracle(built_lib, order, precision):
    ctx, n = _cube(order, precision)
    rng = np.random.default_rng(order)
    pts = rng.uniform(5.0, 395.0, (12, 3))
    coords, material, _ = ctx.get_geometry()
    c3, _ = receivers.locate(coords, pts[3:4])
    pts = np.vstack([pts, coords[c3[0]].mean(axis=0), [100.0, 100.0, 100.0]])  # a second point in one cell; a vertex
    q0 = seeded_dofs(n, order, 4)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    cells = ctx.receivers_setup(pts, dt / 3.0, rotation=True, strain=True)
    ref_cells, xez = receivers.locate(coords, pts)
    assert np.array_equal(cells, ref_cells)
    assert cells[12] == cells[3]
    star = ctx.get_cells()["star"].astype(np.float64)
    o = oracle_py.Oracle(order)
    coeffs = dg_setup.taylor_integrate(order, 0.0, dt)
    times = _times(0.0, dt / 3.0, dt, 4)
    want = []
    for s in range(4):
        q = ctx.get_dofs()
        _, d = o.ader(q.astype(np.float64), star, coeffs, want_derivs=True)
        T = s * dt
        rows = []
        for r in range(len(pts)):
            phi, dphi = receivers.basis_at(order, xez[r], coords[cells[r]])
            rr = receivers.sample(order, d[cells[r]], phi, dphi, [t - T for t in times[s]], rotation=True, strain=True)
            rr[:, 0] += T
            rows.append(rr)
        want.append(np.stack(rows, axis=1))  # [samples, receivers, columns]
        ctx.run("all", dt, 1)
    ctx.sync()
    want = np.concatenate(want)
    got = ctx.receivers_read()
    assert got.shape == want.shape == (sum(len(t) for t in times), len(pts), 1 + 9 + 3 + 6)
    assert np.array_equal(got[:, :, 0], np.broadcast_to(np.concatenate(times)[:, None], got.shape[:2]))
    scale = np.abs(want).max(axis=(0, 1))
    err = np.abs(got - want).max(axis=(0, 1)) / np.maximum(scale, 1e-30)
    assert err[1:].max() < 2e-5, err
    assert abs(ctx.time() - 4 * dt) < 1e-15
    ctx.close()


def test_receiver_staging_many_samples(built_lib):
    ctx, n = _cube(4)
    ctx.set_dofs(seeded_dofs(n, 4, 6))
    dt = ctx.cfl_timestep(0.5)
    pts = np.array([[50.0, 60.0, 70.0], [210.0, 120.0, 330.0], [390.0, 10.0, 200.0]])
    ctx.receivers_setup(pts, dt / 40.0, quantities=[6, 7, 8])
    ctx.run("all", dt, 30)
    first = ctx.receivers_read()
    ctx.run("all", dt, 30)
    second = ctx.receivers_read()
    times = np.concatenate(_times(0.0, dt / 40.0, dt, 60))
    got = np.concatenate([first, second])
    assert got.shape == (len(times), 3, 4)
    assert np.array_equal(got[:, 0, 0], times) and np.array_equal(got[:, 2, 0], times)
    assert len(first) == sum(len(t) for t in _times(0.0, dt / 40.0, dt, 30))
    assert np.isfinite(got).all()
    assert len(ctx.receivers_read()) == 0
    ctx.close()


def test_fault_snapshots_equal_state(built_lib):
    from seissol_gb300 import LSWParams
    ctx, n = _cube(4, fault_plane=2)
    nf = ctx.dr_setup_lsw(LSWParams.fault_config(seed=3))
    tf = np.full((nf, 25), 1e300)
    tf[: nf // 2] = 0.0
    ctx.dr_set_state("forced_rupture_time", tf)
    ctx.set_dofs(seeded_dofs(n, 4, 8))
    fields = ["slip_rate1", "slip", "rupture_time", "mu"]
    ctx.fault_output_setup(2, fields)
    dt = ctx.cfl_timestep(0.5)
    direct = []
    for s in range(6):
        ctx.run("all_dr", dt, 1)
        ctx.sync()
        if s % 2 == 1:
            direct.append((ctx.dr_time(), np.stack([ctx.dr_state(f) for f in fields])))
    times, snaps = ctx.fault_output_read()
    assert len(times) == 3
    for k, (t, st) in enumerate(direct):
        assert times[k] == t
        assert np.array_equal(snaps[k], st)
    assert (snaps[-1][2] >= 0).any()  # ruptured points carry their rupture time
    ctx.close()


def test_output_errors(built_lib):
    from seissol_gb300 import SeiError
    ctx, n = _cube(4)
    with pytest.raises(SeiError) as e:
        ctx.receivers_setup([[1e5, 0.0, 0.0]], 1e-3)
    assert e.value.code == -1 and "outside" in str(e.value)
    with pytest.raises(SeiError) as e:
        ctx.fault_output_setup(1, ["slip"])
    assert e.value.code == -6
    ctx.receivers_setup([[10.0, 10.0, 10.0]], 1e-3)
    ctx.receivers_setup([], 1e-3)  # removes them
    assert ctx.lib.sei_receivers_columns(ctx.h) == 0
    ctx.close()



def test_receivers_under_lts_match_oracle(built_lib):
    """Graded cube in several rate-2 clusters, 10 receivers sampled every 0.73 dt0 over two
    cycles: each cluster samples its receivers at the start of its own steps; against the LTS
    restatement (FP64 trajectory, so 1e-4 of each column's largest magnitude); times exact.
    The interval keeps samples off the step boundaries: a sample on a boundary belongs to one
    step or the next depending on the last bit of the step time, and the predictor's value at a
    step's end differs from the corrected one at the next step's start.  Receivers set before
    the LTS set-up are located again on the reordered cells."""
    from tests.test_gpu_lts import _graded_ctx
    order = 4
    ctx, n = _graded_ctx(order)
    coords0, _, _ = ctx.get_geometry()
    lo, hi = coords0.min(axis=(0, 1)), coords0.max(axis=(0, 1))
    pts = lo + (hi - lo) * np.random.default_rng(3).uniform(0.05, 0.95, (10, 3))
    ctx.receivers_setup(pts, 1e-3)
    ncl = ctx.lts_setup(0.5, 8)
    assert ncl >= 2 and ctx.lib.sei_receivers_columns(ctx.h) == 1 + 9
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    vp = np.sqrt((material[:, 2] + 2 * material[:, 1]) / material[:, 0])
    cl, dt0 = oracle_py.lts_clusters(dg_setup.cfl_timestep(coords, vp, order, 0.5), cells["neighbor"],
                                     cells["face_type"], 8)
    interval = 0.73 * dt0
    rc = ctx.receivers_setup(pts, interval, rotation=True)
    ref_cells, xez = receivers.locate(coords, pts)
    assert np.array_equal(rc, ref_cells)
    assert len(set(cl[rc])) >= 2  # receivers in more than one cluster
    q0 = seeded_dofs(n, order, 5)
    ctx.set_dofs(q0)
    ctx.lts_run(2)
    ctx.sync()
    got = ctx.receivers_read()
    # the restatement, sampled at each cluster's predictor
    o = oracle_py.Oracle(order)
    star = cells["star"].astype(np.float64)
    times = [0.0]
    cursor = {}
    samples = {}

    def t_of(k):
        while len(times) <= k:
            times.append(times[-1] + interval)
        return times[k]

    def on_predict(c, T, dtc, Q):
        recs = [r for r in range(len(pts)) if cl[rc[r]] == c]
        k = cursor.get(c, 0)
        ks = []
        while recs and t_of(k) < T + dtc:
            ks.append(k)
            k += 1
        cursor[c] = k
        if not ks:
            return
        _, d = o.ader(np.asarray(Q, np.float64)[rc[recs]], star[rc[recs]],
                      dg_setup.taylor_integrate(order, 0.0, dtc), want_derivs=True)
        for j, r in enumerate(recs):
            phi, dphi = receivers.basis_at(order, xez[r], coords[rc[r]])
            rows = receivers.sample(order, d[j], phi, dphi, [t_of(k) - T for k in ks], rotation=True)
            rows[:, 0] += T
            for k, row in zip(ks, rows):
                samples.setdefault(k, {})[r] = row

    oracle_py.lts_cycles(o, q0, cells, cl, dt0, 2, on_predict=on_predict)
    complete = []
    for k in range(len(times)):
        if len(samples.get(k, {})) < len(pts):
            break
        complete.append(np.stack([samples[k][r] for r in range(len(pts))]))
    want = np.stack(complete)
    assert got.shape == want.shape, (got.shape, want.shape)
    assert np.array_equal(got[:, :, 0], want[:, :, 0])
    scale = np.abs(want).max(axis=(0, 1))
    err = np.abs(got - want).max(axis=(0, 1)) / np.maximum(scale, 1e-30)
    assert err[1:].max() < 1e-4, err
    ctx.close()


@pytest.mark.parametrize("order", [4, 5])
def test_viscoelastic_receivers_match_oracle(built_lib, order):
    """The nine elastic quantities of the viscoelastic equations (3 mechanisms) at 8 receivers, 3
    samples per step over 3 steps, each step from the GPU's DOFs at its start through the dense
    FP64 viscoelastic predictor; 2e-5 of each column's largest magnitude, times exact."""
    from seissol_gb300 import Context
    from oracle import visco
    QP, QS, FC, RATIO = 50.0, 25.0, 1.0, 100.0
    ctx = Context(order, device=0)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.05, seed=2)
    ctx.visco_setup(QP, QS, FC, RATIO)
    coords, material, _ = ctx.get_geometry()
    cells = ctx.get_cells()
    mats, thetas = [], []
    for rho, mu, lam in material:
        mu_u, lam_u, omega, theta = visco.fit_attenuation(rho, mu, lam, QP, QS, FC, RATIO)
        mats.append([rho, mu_u, lam_u])
        thetas.append(theta)
    ops = visco.cell_operators(coords, np.array(mats), omega, np.array(thetas), cells["neighbor"])
    star = np.concatenate([ops["star"], ops["ET"][:, None]], axis=1)
    pts = np.random.default_rng(order).uniform(5.0, 395.0, (8, 3))
    q0 = np.random.default_rng(7).uniform(-1, 1, (n, 27, ctx.B)).astype(np.float32)
    ctx.set_dofs(q0)
    dt = ctx.cfl_timestep(0.5)
    rc = ctx.receivers_setup(pts, dt / 3.0, rotation=True, strain=True)
    ref_cells, xez = receivers.locate(coords, pts)
    assert np.array_equal(rc, ref_cells)
    o = visco.ViscoLts(order)
    times = _times(0.0, dt / 3.0, dt, 3)
    want = []
    for s in range(3):
        q = ctx.get_dofs()
        _, d = o.ader(q[rc].astype(np.float64), star[rc], dg_setup.taylor_integrate(order, 0.0, dt), want_derivs=True)
        T = s * dt
        rows = []
        for r in range(len(pts)):
            phi, dphi = receivers.basis_at(order, xez[r], coords[rc[r]])
            rr = receivers.sample(order, d[r], phi, dphi, [t - T for t in times[s]], rotation=True, strain=True,
                                  visco=True)
            rr[:, 0] += T
            rows.append(rr)
        want.append(np.stack(rows, axis=1))
        ctx.run("all", dt, 1)
    ctx.sync()
    want = np.concatenate(want)
    got = ctx.receivers_read()
    assert got.shape == want.shape
    assert np.array_equal(got[:, :, 0], want[:, :, 0])
    scale = np.abs(want).max(axis=(0, 1))
    err = np.abs(got - want).max(axis=(0, 1)) / np.maximum(scale, 1e-30)
    assert err[1:].max() < 2e-5, err
    ctx.close()
