"""Regenerate the golden fixtures in this folder from the reference's own files.

Run in a checkout that has the reference source tree (default location given by
``--reference``).  It reads files as text only; nothing of the reference is
compiled or imported.  Outputs:

* ``godunov_elastic.json``  -- Godunov-state matrices of ``tests/Model/Values.h``
  (homogeneous and heterogeneous elastic cases, free-surface boundary) with the two materials.
* ``basis_functions.json`` -- basis-function values and reference-coordinate derivatives at
  (0.3, 0.3, 0.3) of ``tests/Numerical/BasisFunctions.t.h``.
* ``dr_matrices_pin.json`` -- for ``codegen/matrices/dr_stroud_matrices_{4,5,6}.json``: the
  quadrature points and weights in full and the same summary as below for V3mTo2n,
  V3mTo2nTWDivM and resample.
* ``plasticity_nb_pin.json`` -- for ``codegen/matrices/plasticity-nb-matrices-{4,5,6}.json``:
  the nodes (vNodes) in full and the same summary as above for v and vInv.
* ``global_matrices_pin.json`` -- for every matrix of
  ``codegen/matrices/matrices_{20,35,56}.xml``: shape, non-zero count, sum,
  Frobenius norm and a deterministic sample of entries.
"""
import argparse
import json
import os
import re
import xml.etree.ElementTree as ET

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_values_h(path):
    text = open(path).read()
    out = {}
    for name in ("SolutionHomogeneousLocal", "SolutionHomogeneousNeighbor",
                 "SolutionHeterogeneousLocal", "SolutionHeterogeneousNeighbor", "SolutionBoundary"):
        m = re.search(name + r"\s*=\s*\{(.*?)\};", text, re.S)
        body = m.group(1)
        rows = []
        for row in re.findall(r"\{([^{}]*)\}", body):
            vals = []
            for tok in row.split(","):
                tok = tok.strip()
                if not tok:
                    continue
                vals.append(float(eval(tok, {"__builtins__": {}})))
            rows.append(vals)
        assert len(rows) == 9 and all(len(r) == 9 for r in rows), name
        out[name] = rows
    m = re.search(r"struct SolutionData<model::ElasticMaterial>.*?MaterialVal1\{([^}]*)\}.*?MaterialVal2\{([^}]*)\}", text, re.S)
    out["MaterialVal1"] = [float(x) for x in m.group(1).split(",")]
    out["MaterialVal2"] = [float(x) for x in m.group(2).split(",")]
    out["_layout"] = "golden[j][i] == QgodView(i, j); materials are (rho, mu, lambda)"
    return out


def parse_basis_tests(path):
    """Values and reference-coordinate derivatives of the basis functions at (0.3, 0.3, 0.3),
    tests/Numerical/BasisFunctions.t.h (orders up to 6: 56 functions)."""
    text = open(path).read()
    num = r"-?[0-9.]+(?:e-?[0-9]+)?"
    i = text.index("precomputedValues", text.index("Sampled Basis Functions"))
    body = text[i: text.index("};", i)]
    values = [float(x) for x in re.findall(num, body[body.index("{"):])]
    j = text.index("precomputedValues", text.index("Sampled Derivatives Functions"))
    body = text[j: text.index("}}};", j) + 4]
    groups = re.findall(r"\{([^{}]*)\}", body)
    derivs = [[float(x) for x in re.findall(num, g)] for g in groups if re.search(num, g)]
    assert len(values) == 56 and len(derivs) == 3 and all(len(d) == 56 for d in derivs)
    return {"point": [0.3, 0.3, 0.3], "values": values, "derivatives": derivs,
            "_layout": "derivatives[direction][function], direction = d/dxi, d/deta, d/dzeta"}


def parse_xml(path):
    root = ET.parse(path).getroot()
    res = {}
    for m in root:
        rows, cols = int(m.get("rows")), int(m.get("columns"))
        ent = [(int(e.get("row")) - 1, int(e.get("column")) - 1, float(e.get("value"))) for e in m]
        ent.sort()
        nz = [e for e in ent if e[2] != 0.0]
        step = max(1, len(nz) // 24)
        res[m.get("name")] = {
            "shape": [rows, cols],
            "nnz": len(nz),
            "sum": sum(e[2] for e in nz),
            "fro": sum(e[2] ** 2 for e in nz) ** 0.5,
            "sample": [[r, c, v] for (r, c, v) in nz[::step]],
        }
    return res


def parse_dr_json(path):
    res = {}
    for m in json.load(open(path)):
        rows, cols = int(m["rows"]), int(m["columns"])
        ent = sorted((int(e[0]) - 1, int(e[1]) - 1, float(e[2])) for e in m["entries"])
        if m["name"] in ("quadpoints", "quadweights"):
            res[m["name"]] = {"shape": [rows, cols], "entries": [[r, c, v] for (r, c, v) in ent]}
            continue
        nz = [e for e in ent if e[2] != 0.0]
        step = max(1, len(nz) // 24)
        res[m["name"]] = {"shape": [rows, cols], "nnz": len(nz), "sum": sum(e[2] for e in nz),
                          "fro": sum(e[2] ** 2 for e in nz) ** 0.5, "sample": [[r, c, v] for (r, c, v) in nz[::step]]}
    return res


def parse_plasticity_json(path):
    res = {}
    for m in json.load(open(path)):
        if m["name"] not in ("vNodes", "v", "vInv"):
            continue
        shape = [int(x) for x in m["shape"]]
        ent = sorted((int(e[0]) - 1, int(e[1]) - 1, float(e[2])) for e in m["entries"])
        if m["name"] == "vNodes":
            full = [[0.0] * shape[1] for _ in range(shape[0])]
            for r, c, v in ent:
                full[r][c] = v
            res["nodes"] = full
            continue
        nz = [e for e in ent if e[2] != 0.0]
        step = max(1, len(nz) // 40)
        res[m["name"]] = {"shape": shape, "nnz": len(nz), "sum": sum(e[2] for e in nz),
                          "fro": sum(e[2] ** 2 for e in nz) ** 0.5, "sample": [[r, c, v] for (r, c, v) in nz[::step]]}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SEI_REFERENCE_ROOT"),
                    help="root of the reference source tree (default: $SEI_REFERENCE_ROOT)")
    a = ap.parse_args()
    if not a.reference:
        ap.error("name the reference tree with --reference or SEI_REFERENCE_ROOT")
    g = parse_values_h(os.path.join(a.reference, "tests/Model/Values.h"))
    json.dump(g, open(os.path.join(HERE, "godunov_elastic.json"), "w"), indent=1)
    json.dump(parse_basis_tests(os.path.join(a.reference, "tests/Numerical/BasisFunctions.t.h")),
              open(os.path.join(HERE, "basis_functions.json"), "w"), indent=1)
    pin = {}
    for b in (20, 35, 56):
        pin[str(b)] = parse_xml(os.path.join(a.reference, f"codegen/matrices/matrices_{b}.xml"))
    json.dump(pin, open(os.path.join(HERE, "global_matrices_pin.json"), "w"))
    dr = {str(o): parse_dr_json(os.path.join(a.reference, f"codegen/matrices/dr_stroud_matrices_{o}.json"))
          for o in (4, 5, 6)}
    json.dump(dr, open(os.path.join(HERE, "dr_matrices_pin.json"), "w"))
    pl = {str(o): parse_plasticity_json(os.path.join(a.reference, f"codegen/matrices/plasticity-nb-matrices-{o}.json"))
          for o in (4, 5, 6)}
    json.dump(pl, open(os.path.join(HERE, "plasticity_nb_pin.json"), "w"))


if __name__ == "__main__":
    main()
