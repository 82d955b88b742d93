"""PUML mesh ingestion, restated (TEST INFRASTRUCTURE ONLY).

Follows src/Geometry/PUMLReader.cpp (cells from the geometry / connect / boundary arrays of
docs/puml-mesh-format.rst, topology from identify-vertex when given), the default face map of
src/Initializer/FaceMap.cpp:100-110 and the fault plus side of src/Geometry/MeshReader.cpp:150-170,
on top of dg_setup's face relations, operators and fault-face data.
"""
import numpy as np

from . import dg_setup

FACE2MISSING = (3, 2, 1, 0)


def decode_boundary(boundary, fmt, n):
    """Boundary condition per (cell, face): i32 8 bits per face, i64 16 bits, i32x4 one value each."""
    if boundary is None:
        return np.zeros((n, 4), dtype=np.int64)
    b = np.asarray(boundary)
    if fmt == "i32x4":
        return b.reshape(n, 4).astype(np.int64)
    bits, mask = (8, 0xFF) if fmt == "i32" else (16, 0xFFFF)
    b = b.astype(np.uint64)
    return np.stack([((b >> np.uint64(bits * f)) & np.uint64(mask)).astype(np.int64) for f in range(4)], axis=1)


def ingest(geometry, connect, material, boundary=None, fmt="i32", identify=None, ref=(0.0, 0.0, 0.0),
           method="point"):
    """Returns dict: topo, coords, neighbor, side, orient, face_type (0 regular, 1 fault,
    2 boundary), bc (1 free surface, 5 outflow), ops (cell_operators), fault (plus_face [nf, 4],
    rel [nf]) and fault_data (fault_face_data)."""
    geometry = np.asarray(geometry, float)
    connect = np.asarray(connect, np.int64)
    material = np.asarray(material, float)
    n = connect.shape[0]
    topo = np.asarray(identify, np.int64)[connect] if identify is not None else connect
    coords = geometry[connect]
    nb, side, orient = dg_setup.face_relations(topo)
    codes = decode_boundary(boundary, fmt, n)
    face_type = np.where(nb >= 0, 0, 2).astype(np.int64)
    bc = np.zeros((n, 4), dtype=np.int64)
    for c in range(n):
        for f in range(4):
            b = codes[c, f]
            if b == 3 or b > 64:
                face_type[c, f] = 1
                face_type[nb[c, f], side[c, f]] = 1
            elif b in (1, 5):
                bc[c, f] = b
    ref = np.asarray(ref, float)
    plus, rel = [], []
    for c in range(n):
        for f in range(4):
            if face_type[c, f] != 1:
                continue
            v = coords[c]
            a, b_, cc = (v[k] for k in dg_setup.FACE2NODES[f])
            nrm = np.cross(b_ - a, cc - a)
            if method == "point":
                s = np.dot(ref - a, nrm) * np.dot(v[FACE2MISSING[f]] - a, nrm)
            else:
                s = np.dot(ref, nrm)
            if s > 0:
                plus.append((c, f, nb[c, f], side[c, f]))
                rel.append(orient[c, f] + 1)
    plus = np.array(plus, dtype=np.int64).reshape(-1, 4)
    ops = dg_setup.cell_operators(coords, material, nb, face_type, bc)
    fd = dg_setup.fault_face_data(coords, material, plus) if len(plus) else None
    return {"topo": topo, "coords": coords, "neighbor": nb, "side": side, "orient": orient,
            "face_type": face_type, "bc": bc, "ops": ops, "fault": {"plus_face": plus, "rel": np.array(rel)},
            "fault_data": fd}
