"""seissol-proxy equivalent over the C ABI.

Mirrors src/Proxy/Common.h:18-48 (ProxyConfig, ProxyOutput), src/Proxy/Runner.cpp:57-152
(one warm-up step, then ``timesteps`` timed steps) and the pybind module
app/Proxy/Bindings.cpp:14-60.  Unlike the reference proxy, the data are a real mesh
(synthetic periodic cube) with physical operators, and the time step is the CFL step.

CLI:  python -m seissol_gb300.proxy <cells> <timesteps> <kernel>[,kernel...] [--order N] [--format json]
      [--precision fp32|f16x3]; the *_dr kernels run on a planar fault at orders 4-6.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import sys
import time

from .lib import KERNELS, Context

# Non-zero flops and algorithmic bytes per cell and step of each proxy kernel; filled from
# the generator's counts at import of the codegen package when available.
_BYTES_PER_CELL = None


@dataclasses.dataclass
class ProxyConfig:
    cells: int = 100000
    timesteps: int = 10
    kernels: tuple = ("all",)
    order: int = 6
    verbose: bool = True
    device: int = 0
    precision: int = 0  # SEI_PREC_FP32 / SEI_PREC_F16X3


@dataclasses.dataclass
class ProxyOutput:
    time: float = 0.0
    cycles: float = 0.0
    actualNonZeroGFlop: float = 0.0
    actualHardwareGFlop: float = 0.0
    gib: float = 0.0
    nonZeroGFlops: float = 0.0
    hardwareGFlops: float = 0.0
    gibPerSecond: float = 0.0
    cellUpdatesPerSecond: float = 0.0


def cube_dims(cells: int):
    """Even cube counts (nx, ny, nz) with 5 nx ny nz >= cells, as cubic as possible."""
    cubes = max(8, math.ceil(cells / 5))
    s = max(2, int(round(cubes ** (1 / 3))))
    s += s % 2
    nx = ny = s
    nz = max(2, math.ceil(cubes / (nx * ny)))
    nz += nz % 2
    return nx, ny, nz


def bytes_per_cell(order: int) -> float:
    """Compulsory HBM bytes of one cell update (ADER + local + neighbour), float32."""
    b = order * (order + 1) * (order + 2) // 6
    return 4.0 * (4 * b * 9 + 3 * 24 + 4 * 81 + 4 * 81) + 4 * 4 + 4 + 4


def run_proxy(cfg: ProxyConfig) -> ProxyOutput:
    for k in cfg.kernels:
        if k not in KERNELS:
            raise ValueError(f"unknown kernel {k}; allowed: {', '.join(KERNELS)}")
    nx, ny, nz = cube_dims(cfg.cells)
    dr = any(k.endswith("_dr") for k in cfg.kernels)
    with Context(cfg.order, cfg.device, precision=cfg.precision) as ctx:
        # the *_dr kernels run on a planar fault through the middle of the cube (x = nx / 2),
        # fast-velocity-weakening friction with the fault parameters of RSParams.fault_config
        n = ctx.build_periodic_cube(nx, ny, nz, fault_plane=nx // 2 if dr else -1)
        if dr:
            from .lib import RSParams
            ctx.dr_setup(RSParams.fault_config())
        dt = ctx.cfl_timestep(0.5)
        for k in cfg.kernels:
            ctx.run(k, dt, 1)  # warm-up
        ctx.sync()
        t0 = time.perf_counter()
        total_ms = 0.0
        for k in cfg.kernels:
            ctx.run(k, dt, cfg.timesteps)
            ctx.sync()
            total_ms += ctx.last_run_ms()
        wall = time.perf_counter() - t0
    try:
        from .codegen.gen_kernels import nnz_flops
        f = nnz_flops(cfg.order)
        per = {"all": f["ader"] + f["local"] + f["neighbor"], "local": f["ader"] + f["local"], "neigh": f["neighbor"],
               "ader": f["ader"], "localwoader": f["local"]}
        flop = sum(per.get(k, 0.0) for k in cfg.kernels) * n * cfg.timesteps
    except Exception:
        flop = 0.0
    secs = total_ms / 1e3 if total_ms > 0 else wall
    gib = bytes_per_cell(cfg.order) * n * cfg.timesteps * len(cfg.kernels) / 2 ** 30
    out = ProxyOutput(time=secs, actualNonZeroGFlop=flop / 1e9, actualHardwareGFlop=flop / 1e9, gib=gib,
                      nonZeroGFlops=flop / 1e9 / secs, hardwareGFlops=flop / 1e9 / secs, gibPerSecond=gib / secs,
                      cellUpdatesPerSecond=n * cfg.timesteps / secs)
    return out


def write_output(out: ProxyOutput, name: str, fmt: str = "plain", stream=sys.stdout):
    if fmt == "json":
        stream.write(json.dumps({"name": name, "time": out.time, "gflop-nz": out.actualNonZeroGFlop,
                                 "gflop-hw": out.actualHardwareGFlop, "gib": out.gib, "gflops-nz": out.nonZeroGFlops,
                                 "gflops-hw": out.hardwareGFlops, "gibs": out.gibPerSecond,
                                 "cell-updates-per-s": out.cellUpdatesPerSecond}) + "\n")
        return
    stream.write("=================================================\n")
    stream.write("===            PERFORMANCE SUMMARY            ===\n")
    stream.write("=================================================\n")
    for label, val in (("seissol proxy mode", name), ("time for seissol proxy", out.time),
                       ("GFLOP (non-zero) for seissol proxy", out.actualNonZeroGFlop),
                       ("GiB (estimate) for seissol proxy", out.gib),
                       ("GFLOPS (non-zero) for seissol proxy", out.nonZeroGFlops),
                       ("GiB/s (estimate) for seissol proxy", out.gibPerSecond),
                       ("cell updates/s", out.cellUpdatesPerSecond)):
        stream.write(f"{label:<36}: {val}\n")
    stream.write("=================================================\n")


def main(argv=None):
    ap = argparse.ArgumentParser(prog="seissol-proxy-gb300")
    ap.add_argument("cells", type=int)
    ap.add_argument("timesteps", type=int)
    ap.add_argument("kernel")
    ap.add_argument("--order", type=int, default=6)
    ap.add_argument("--format", choices=("plain", "json"), default="plain")
    ap.add_argument("--precision", choices=("fp32", "f16x3"), default="fp32",
                    help="f16x3: the tensor-core path (split FP16 x3 contractions, FP32 accumulation)")
    a = ap.parse_args(argv)
    kernels = tuple(a.kernel.split(","))
    out = run_proxy(ProxyConfig(cells=a.cells, timesteps=a.timesteps, kernels=kernels, order=a.order,
                                precision={"fp32": 0, "f16x3": 1}[a.precision]))
    write_output(out, a.kernel, a.format)
    return 0


if __name__ == "__main__":
    sys.exit(main())
