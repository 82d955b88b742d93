"""In-tree build of libsei_gb300.so for sm_103a.

Steps: generate the per-order kernel bodies (seissol_gb300/codegen), compile every
translation unit with nvcc in parallel (one -gencode, sm_103a), link one shared library
next to this file.  Rebuilds only what changed (source or generated header newer than
the object).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
GEN = os.path.join(CSRC, "_gen")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsei_gb300.so")
ORDERS = (4, 5, 6)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sei_gb300")


def _sources():
    srcs = [os.path.join(CSRC, f"kernels_o{o}.cu") for o in ORDERS]
    srcs += [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu") and not f.startswith("kernels_o")]
    srcs += [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cpp")]
    return srcs


def _deps(src):
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "sei_gb300.h"))
    base = os.path.basename(src)
    if base.startswith("kernels_"):
        deps.append(os.path.join(GEN, base.replace(".cu", ".cuh")))
    if base.startswith("dr_"):
        deps += [os.path.join(GEN, f"dr_tables_o{o}.cuh") for o in ORDERS]
    if base.startswith("tc_"):
        deps += [os.path.join(GEN, f"{n}_o{o}.cuh") for n in ("tc_tables", "tc_nb") for o in ORDERS]
    return deps


def _compile(src, verbose=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in _deps(src) if os.path.exists(d)):
        return obj, ""
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "--expt-relaxed-constexpr",
               "-Xptxas", "-v", *inc, "-c", src, "-o", obj]
    else:
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", *inc, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    sys.path.insert(0, ROOT)
    from seissol_gb300.codegen import gen_kernels, gen_visco

    os.makedirs(OBJ, exist_ok=True)
    gen_kernels.write_all(GEN, ORDERS)
    gen_visco.write_all(GEN)
    gen_kernels.write_dr_tables(GEN, ORDERS)
    gen_kernels.write_tc_tables(GEN, ORDERS)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for (o, log) in results:
            if log:
                print(f"--- {os.path.basename(o)}\n{log}")
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
