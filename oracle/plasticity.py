"""Off-fault plasticity restated in float64 numpy.  Test infrastructure (the checker): only tests,
the smoke check and the CPU legs of the benchmark use it.

Follows src/Kernels/Plasticity.cpp:47-214 (computePlasticity), src/Kernels/Plasticity.h:27-29
(computeRelaxTime) and src/Model/Plasticity.h:28-59 (PlasticityData):
* the modal stresses go to the nodes through V (the basis functions at the nodes), plus the
  initial loading;
* at each node: the mean stress m, the deviator s, tau = sqrt(J2) with J2 = s_ij s_ij / 2, and
  tau_c = max(0, c cos(phi) - m sin(phi)), phi = atan(bulk friction);
* where tau > tau_c the yield factor is (tau_c / tau - 1) r, r = 1 - exp(-dt / T_v); the stress
  update is the deviator times it, the plastic strain integrates -1 / (2 mu T_v r) times the
  update (explicit Euler) and eta the norm sqrt(e_ij e_ij / 2) of that rate;
* a cell with a yielding node adds Vinv times the nodal update to its modal stresses.
Parity pins: V and Vinv at the reference's nodes against its plasticity-nb matrices (fixture
tests/golden/plasticity_nb_pin.json) and computeRelaxTime's known answers
(tests/Kernel/Plasticity.t.h).
"""
import numpy as np

from . import dg_setup


def relax_factor(tv, dt):
    """computeRelaxTime (Plasticity.h:27-29)."""
    return float(-np.expm1(-dt / tv)) if tv > 0.0 else 1.0


def lattice_nodes(order):
    """The equispaced lattice of degree order - 1 (i fastest), the library's default node set."""
    d = order - 1
    pts = [(i / d, j / d, k / d) for k in range(d + 1) for j in range(d + 1 - k) for i in range(d + 1 - j - k)]
    return np.array(pts, np.float64)


def matrices(order, nodes):
    """V [nodes, B] (phi_k at node n) and its inverse [B, nodes]."""
    x = np.asarray(nodes, np.float64)
    cols = [np.real(dg_setup.tet_dubiner(i, j, k, x[:, 0], x[:, 1], x[:, 2]))
            for (i, j, k) in dg_setup.basis_indices3(order)]
    v = np.stack(cols, axis=1)
    return v, np.linalg.inv(v)


def cell_parameters(bulk_friction, plast_co, s0, nnodes, per_node=False):
    """PlasticityData of every cell: s0 [n, 6, B], c cos(phi) and sin(phi) [n, B]."""
    bf, co, s0 = (np.asarray(a, np.float64) for a in (bulk_friction, plast_co, s0))
    if not per_node:
        bf = np.repeat(bf[:, None], nnodes, axis=1)
        co = np.repeat(co[:, None], nnodes, axis=1)
        s0 = np.repeat(s0[:, None, :], nnodes, axis=1)
    phi = np.arctan(bf)
    return np.transpose(s0, (0, 2, 1)).copy(), co * np.cos(phi), np.sin(phi)


def apply(q, pstrain, v, vinv, s0, ccos, ssin, mu, dt, tv):
    """One plasticity update of every cell, in place.  q [n, 9, >= B] modal DOFs, pstrain [n, 7, B];
    s0 [n, 6, B], ccos and ssin [n, B], mu [n].  Returns the yielding cells (bool [n])."""
    B = v.shape[1]
    r = relax_factor(tv, dt)
    nodal = np.einsum("nk,cxk->cxn", v, q[:, :6, :B]) + s0
    m = nodal[:, :3].mean(axis=1)
    dev = nodal.copy()
    dev[:, :3] -= m[:, None, :]
    j2 = 0.5 * (dev[:, :3] ** 2).sum(axis=1) + (dev[:, 3:] ** 2).sum(axis=1)
    tau = np.sqrt(j2)
    lim = np.maximum(0.0, ccos - m * ssin)
    yielding = tau > lim
    y = np.where(yielding, (np.divide(lim, tau, out=np.ones_like(tau), where=yielding) - 1.0) * r, 0.0)
    upd = dev * y[:, None, :]
    rate = -(1.0 / (2.0 * mu) / (tv * r))[:, None, None] * upd
    adjust = yielding.any(axis=1)
    pstrain[adjust, :6] += dt * rate[adjust]
    pstrain[adjust, 6] += dt * np.sqrt(0.5 * (rate[adjust] ** 2).sum(axis=1))
    q[adjust, :6, :B] += np.einsum("kn,cxn->cxk", vinv, upd[adjust])
    return adjust
