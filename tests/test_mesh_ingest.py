"""PUML mesh ingestion (sei_set_mesh) against its restatement and the reference's pins (CPU only).

* free-surface Godunov state vs SolutionBoundary of tests/Model/Values.h (fixture
  godunov_elastic.json), tolerance 1e-15 absolute on entries of order 1e-7 and 1;
* a 4 x 4 x 4 box (320 tets, heterogeneous material) with a free-surface top, outflow sides and
  two crossing fault planes (tags 3 and 65): face relations, face types, fault faces (plus side
  by a reference point and by a reference normal) exact; operators, TinvT, flux solvers and
  impedances within float32 rounding (2e-6 relative to each matrix's largest entry);
* the three boundary formats decode alike;
* a periodic cube given as geometric vertices plus identify-vertex equals the built-in cube bit
  for bit;
* malformed meshes are rejected with the error the ABI documents and leave the context as it was.
"""
import json
import os

import numpy as np
import pytest

from oracle import cube_mesh, dg_setup, puml

HERE = os.path.dirname(os.path.abspath(__file__))
SEI_ERR_ARG, SEI_ERR_UNSUPPORTED = -1, -7


def _material(n, seed=3):
    rng = np.random.default_rng(seed)
    rho = 2700.0 * rng.uniform(0.9, 1.1, n)
    vs = 3464.0 * rng.uniform(0.9, 1.1, n)
    vp = 6000.0 * rng.uniform(0.9, 1.1, n)
    mu = rho * vs * vs
    return np.stack([rho, mu, rho * vp * vp - 2 * mu], axis=1)


def _host():
    from seissol_gb300 import Context
    return Context(4, device=-1)


def test_free_surface_state_pinned():
    g = json.load(open(os.path.join(HERE, "golden", "godunov_elastic.json")))
    q, _ = dg_setup.free_surface_state(g["MaterialVal1"])
    gold = np.array(g["SolutionBoundary"]).T  # golden[j][i] == QgodView(i, j)
    assert np.abs(q - gold).max() < 1e-15


def _close(a, b, tol=2e-6):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.abs(b).reshape(b.shape[0], -1).max(axis=1).reshape((-1,) + (1,) * (b.ndim - 1))
    return (np.abs(a - b) <= tol * np.maximum(scale, 1e-300)).all()


@pytest.mark.parametrize("method,ref", [("point", (-1e4, 0.0, 0.0)), ("normal", (1.0, 1.0, 0.0))])
def test_box_mesh_matches_oracle(built_lib, method, ref):
    geo, con, bnd = cube_mesh.box_mesh(4, 4, 4, fault_x=2, fault_y=2)
    mat = _material(len(con))
    ctx = _host()
    n, nf = ctx.set_mesh(geo, con, mat, boundary=bnd, fault_ref=ref, fault_ref_method=method)
    want = puml.ingest(geo, con, mat, bnd, "i32", None, ref, method)
    assert n == len(con) and nf == len(want["fault"]["plus_face"]) > 0
    cells = ctx.get_cells()
    nb = np.where(want["neighbor"] >= 0, want["neighbor"], -1)
    assert np.array_equal(cells["neighbor"], nb)
    bnd_face = want["neighbor"] < 0
    assert np.array_equal(cells["side"][~bnd_face], want["side"][~bnd_face])
    assert np.array_equal(cells["orient"][~bnd_face], want["orient"][~bnd_face])
    assert np.array_equal(cells["face_type"], want["face_type"])
    assert (want["bc"] == 1).any() and (want["bc"] == 5).any()
    for k in ("star", "AplusT", "AminusT"):
        a = cells[k].reshape(-1, 9, 9)
        b = want["ops"][k].reshape(-1, 9, 9)
        if k == "AminusT":  # boundary faces have no neighbour flux: their A- is not used
            keep = ~bnd_face.reshape(-1)
            a, b = a[keep], b[keep]
        assert _close(a, b), k
    faces = ctx.dr_faces()
    pf = want["fault"]["plus_face"]
    assert np.array_equal(faces["cells"], pf[:, [0, 2]])
    assert np.array_equal(faces["sides"][:, :2], pf[:, [1, 3]])
    assert np.array_equal(faces["sides"][:, 2], want["fault"]["rel"])
    fd = want["fault_data"]
    for k in ("TinvT", "fluxSolverPlus", "fluxSolverMinus"):
        assert _close(faces[k], fd[k]), k
    assert np.allclose(faces["imp"][:, :7], fd["imp"], rtol=1e-12)
    # cells on the crossing line carry two fault faces
    counts = np.bincount(np.concatenate([pf[:, 0], pf[:, 2]]), minlength=n)
    assert counts.max() == 2
    ctx.close()


def test_plus_side_flips_with_the_reference(built_lib):
    geo, con, bnd = cube_mesh.box_mesh(4, 4, 4, fault_x=2)
    mat = _material(len(con))
    a, b = _host(), _host()
    a.set_mesh(geo, con, mat, boundary=bnd, fault_ref=(-1e4, 0, 0))
    b.set_mesh(geo, con, mat, boundary=bnd, fault_ref=(1e4, 0, 0))
    fa, fb = a.dr_faces()["cells"], b.dr_faces()["cells"]
    assert sorted(map(tuple, fa)) == sorted(map(tuple, fb[:, ::-1]))
    # plus side of the first: the cell at x < 2 h
    coords = geo[con]
    assert (coords[fa[:, 0]].mean(axis=1)[:, 0] < 200.0).all()
    a.close()
    b.close()


def test_boundary_formats_agree(built_lib):
    geo, con, bnd = cube_mesh.box_mesh(4, 4, 4, fault_x=2, fault_y=2)
    mat = _material(len(con))
    codes = puml.decode_boundary(bnd.astype(np.uint32), "i32", len(con))
    codes[codes == 3] = 300  # i32 holds 8 bits: tag 300 needs the wider formats
    i64 = np.zeros(len(con), np.uint64)
    for f in range(4):
        i64 |= codes[:, f].astype(np.uint64) << np.uint64(16 * f)
    out = []
    for fmt, arr in (("i64", i64), ("i32x4", codes.astype(np.int32))):
        ctx = _host()
        n, nf = ctx.set_mesh(geo, con, mat, boundary=arr, boundary_format=fmt, fault_ref=(-1e4, 0, 0))
        out.append((nf, ctx.get_cells()["face_type"], ctx.dr_faces()["cells"]))
        ctx.close()
    assert out[0][0] == out[1][0] > 0
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])


def test_periodic_identify_equals_builtin_cube(built_lib):
    a = _host()
    a.build_periodic_cube(4, 4, 4, perturb=0.05, seed=5)
    coords, material, topo = a.get_geometry()
    n = coords.shape[0]
    geo = coords.reshape(-1, 3)
    con = np.arange(4 * n, dtype=np.int64).reshape(n, 4)
    identify = np.empty(4 * n, np.int64)
    identify[con.reshape(-1)] = topo.reshape(-1)
    b = _host()
    b.set_mesh(geo, con, material, identify=identify)
    ca, cb = a.get_cells(), b.get_cells()
    for k in ca:
        assert np.array_equal(ca[k], cb[k]), k
    a.close()
    b.close()


def _err(ctx, **kw):
    from seissol_gb300 import SeiError
    with pytest.raises(SeiError) as e:
        ctx.set_mesh(**kw)
    return e.value


def test_rejected_meshes(built_lib):
    geo, con, bnd = cube_mesh.box_mesh(4, 4, 4, fault_x=2)
    mat = _material(len(con))
    ctx = _host()
    n, nf = ctx.set_mesh(geo, con, mat, boundary=bnd, fault_ref=(-1e4, 0, 0))
    before = ctx.get_cells()
    base = dict(geometry=geo, connect=con, material=mat, boundary=bnd, fault_ref=(-1e4, 0, 0))
    # gravity free surface, Dirichlet, analytical: not supported
    for code in (2, 4, 7):
        b = bnd.copy()
        top = puml.decode_boundary(b, "i32", len(con)) == 1
        c, f = np.argwhere(top)[0]
        b[c] = (b[c] & ~np.uint32(0xFF << (8 * f))) | np.uint32(code << (8 * f))
        e = _err(ctx, **{**base, "boundary": b})
        assert e.code == SEI_ERR_UNSUPPORTED and "not supported" in str(e)
    # no boundary conditions: mesh boundary left open
    e = _err(ctx, **{**base, "boundary": None})
    assert e.code == SEI_ERR_ARG and "without" in str(e)
    # a flipped tetrahedron
    bad = con.copy()
    bad[0, [2, 3]] = bad[0, [3, 2]]
    assert "oriented" in str(_err(ctx, **{**base, "connect": bad}))
    # vertex id out of range, negative density
    bad = con.copy()
    bad[1, 0] = len(geo)
    assert "range" in str(_err(ctx, **{**base, "connect": bad}))
    m2 = mat.copy()
    m2[5, 0] = -1.0
    assert "material" in str(_err(ctx, **{**base, "material": m2}))
    # a reference point on the fault plane decides no side
    assert "side" in str(_err(ctx, **{**base, "fault_ref": (200.0, 50.0, 50.0)}))
    # nothing changed
    after = ctx.get_cells()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    assert ctx.lib.sei_dr_num_faces(ctx.h) == nf
    ctx.close()
