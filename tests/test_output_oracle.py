"""Receiver building blocks pinned to the reference's unit tests (CPU only).

* basis functions and their reference-coordinate derivatives at (0.3, 0.3, 0.3), orders 1-6, vs
  tests/Numerical/BasisFunctions.t.h (fixture basis_functions.json): the oracle's (complex step)
  and the product's (sei_basis_functions, dual numbers), 1e-13 absolute;
* the global-to-reference map of a tetrahedron's centre is (1/4, 1/4, 1/4)
  (tests/Numerical/Transformations.t.h), 10 eps.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from oracle import dg_setup, receivers

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "basis_functions.json")))
REF_TET = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_oracle_basis_pinned(order):
    B = dg_setup.nbasis3(order)
    phi, dphi = receivers.basis_at(order, GOLD["point"], REF_TET)
    assert np.abs(phi - np.array(GOLD["values"][:B])).max() < 1e-13
    assert np.abs(dphi - np.array([d[:B] for d in GOLD["derivatives"]])).max() < 1e-13


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6])
def test_product_basis_pinned(built_lib, order):
    from seissol_gb300 import load_library
    lib = load_library()
    B = dg_setup.nbasis3(order)
    x = np.array(GOLD["point"])
    phi = np.empty(B)
    dphi = np.empty(3 * B)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    assert lib.sei_basis_functions(order, p(x), p(phi), p(dphi)) == 0
    assert np.abs(phi - np.array(GOLD["values"][:B])).max() < 1e-13
    assert np.abs(dphi.reshape(3, B) - np.array([d[:B] for d in GOLD["derivatives"]])).max() < 1e-13


def test_centre_maps_to_quarter():
    rng = np.random.default_rng(9)
    v = rng.uniform(0.0, 1.0, (4, 3))
    if np.linalg.det(np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]])) < 0:
        v[[2, 3]] = v[[3, 2]]
    cells, xez = receivers.locate(v[None], v.mean(axis=0)[None])
    assert cells[0] == 0
    assert np.abs(xez[0] - 0.25).max() < 10 * np.finfo(float).eps
