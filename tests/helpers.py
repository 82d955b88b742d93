"""Shared helpers of the test-suite: relative errors and oracle inputs from a product mesh."""
import numpy as np

from oracle import dg_setup


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def rel_l2_per_quantity(a, b):
    """Relative L2 error of each of the 9 quantities of [n, 9, B] tensors."""
    return [rel_l2(a[:, q], b[:, q]) for q in range(a.shape[1])]


def oracle_inputs_from_geometry(coords, material, topo):
    """Face relations and operators computed by the oracle from the product's geometry."""
    nb, side, orient = dg_setup.face_relations(topo)
    ops = dg_setup.cell_operators(coords, material, nb)
    return nb, side, orient, ops


def seeded_dofs(n, order, seed=7):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, size=(n, 9, dg_setup.nbasis3(order))).astype(np.float32)
