"""seissol-proxy equivalent over the C ABI.

Mirrors src/Proxy/Common.h:18-48 (ProxyConfig, ProxyOutput), src/Proxy/Runner.cpp:57-152
(one warm-up step, then ``timesteps`` timed steps) and the pybind module
app/Proxy/Bindings.cpp:14-60.  Unlike the reference proxy, the data are a real mesh
(synthetic periodic cube) with physical operators, and the time step is the CFL step.

CLI:  python -m seissol_gb300.proxy <cells> <timesteps> <kernel>[,kernel...] [--order N] [--format json]
      [--precision fp32|f16x3] [--mechanisms 0|3] [--plasticity]; the *_dr kernels run on a planar fault at orders
      4-6; --mechanisms 3 runs the viscoelastic equations (orders 4-5), as the reference's proxy
      built for them (Qp 100, Qs 50, central frequency 0.5 Hz, frequency ratio 100).
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
    mechanisms: int = 0  # 0 elastic, 3 viscoelastic (27 quantities)
    plasticity: bool = False  # off-fault plasticity on every cell (elastic, orders 4-6)


@dataclasses.dataclass
class ProxyOutput:
    """The fields of src/Proxy/Common.h:30-48.  The LIBXSMM and PSpaMM counts stay 0: no code of
    those generators runs here.  cycles = time x the device's maximum SM clock (the reference
    counts host cycles, src/Proxy/Runner.cpp:87-129); gib is the compulsory-traffic estimate of the
    step, kernelGib the sum over the launched kernels' own compulsory bytes."""
    time: float = 0.0
    cycles: float = 0.0
    libxsmmNumTotalGFlop: float = 0.0
    pspammNumTotalGFlop: float = 0.0
    libxsmmAndpspammNumTotalGFlop: float = 0.0
    actualNonZeroGFlop: float = 0.0
    actualHardwareGFlop: float = 0.0
    gib: float = 0.0
    kernelGib: float = 0.0
    nonZeroFlopPerCycle: float = 0.0
    hardwareFlopPerCycle: float = 0.0
    bytesPerCycle: float = 0.0
    kernelBytesPerCycle: float = 0.0
    nonZeroGFlops: float = 0.0
    hardwareGFlops: float = 0.0
    gibPerSecond: float = 0.0
    kernelGibPerSecond: float = 0.0
    cellUpdatesPerSecond: float = 0.0

    # the snake_case names of the reference's Python module (app/Proxy/Bindings.cpp:33-51)
    libxsmm_num_total_gflop = property(lambda self: self.libxsmmNumTotalGFlop)
    pspamm_num_total_gflop = property(lambda self: self.pspammNumTotalGFlop)
    libxsmm_and_pspamm_num_total_gflop = property(lambda self: self.libxsmmAndpspammNumTotalGFlop)
    actual_non_zero_gflop = property(lambda self: self.actualNonZeroGFlop)
    actual_hardware_gflop = property(lambda self: self.actualHardwareGFlop)
    non_zero_flop_per_cycle = property(lambda self: self.nonZeroFlopPerCycle)
    hardware_flop_per_cycle = property(lambda self: self.hardwareFlopPerCycle)
    bytes_per_cycle = property(lambda self: self.bytesPerCycle)
    non_zero_gflops = property(lambda self: self.nonZeroGFlops)
    hardware_gflops = property(lambda self: self.hardwareGFlops)
    gib_per_second = property(lambda self: self.gibPerSecond)


class Aux:
    """Kernel-name helpers and output of the proxy (src/Proxy/Common.h:50-62, Common.cpp)."""

    @staticmethod
    def str_to_kernel(kernel_str: str) -> list:
        """'all,neigh' -> ['all', 'neigh']; an unknown name raises ValueError (the reference throws)."""
        parts = [p.strip() for p in kernel_str.split(",")]
        for p in parts:
            if p not in KERNELS:
                raise ValueError(f"Unknown kernel string: {p}")
        return parts

    @staticmethod
    def kernel_to_string(kernels) -> str:
        for k in kernels:
            if k not in KERNELS:
                raise ValueError("Unknown kernel type")
        return ",".join(kernels)

    @staticmethod
    def get_allowed_kernels() -> list:
        return list(KERNELS)

    @staticmethod
    def write_output(stream, out: "ProxyOutput", kernel_str: str, fmt: str = "plain"):
        write_output(out, kernel_str, fmt, stream)

    @staticmethod
    def display_output(out: "ProxyOutput", kernel_str: str):
        write_output(out, kernel_str, "plain", sys.stdout)


def cube_dims(cells: int):
    """Even cube counts (nx, ny, nz) with 5 nx ny nz >= cells, as cubic as possible."""
    cubes = max(8, math.ceil(cells / 5))
    s = max(2, int(round(cubes ** (1 / 3))))
    s += s % 2
    nx = ny = s
    nz = max(2, math.ceil(cubes / (nx * ny)))
    nz += nz % 2
    return nx, ny, nz


def bytes_per_cell(order: int, mechanisms: int = 0) -> float:
    """Compulsory HBM bytes of one cell update (ADER + local + neighbour), float32.  With
    mechanisms: Q read and written, I written and read back, per face the elastic and memory
    blocks of both flux matrices, the star non-zeros, gradients and theta."""
    b = order * (order + 1) * (order + 2) // 6
    if mechanisms:
        nq = 9 + 6 * mechanisms
        return 4.0 * (4 * b * nq + 4 * 2 * (81 + 9 * 6) + 72 + 9 + 9) + 4 * 4 + 4 + 4
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
        if cfg.mechanisms:
            ctx.visco_setup(100.0, 50.0, 0.5, 100.0)
        if cfg.plasticity:
            # bulk friction 0.6, c cos(phi) ~ U[0.7, 1.5] x 87 MPa, initial stress U[-1, 1] MPa,
            # T_v 0.05 s, the library's default nodes
            import numpy as np
            rng = np.random.default_rng(1)
            ctx.plasticity_setup(np.full(n, 0.6), rng.uniform(0.7, 1.5, n) * 8.7e7 / np.cos(np.arctan(0.6)),
                                 rng.uniform(-1e6, 1e6, (n, 6)), tv=0.05)
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
        perf = {}
        for k in ("ader", "localwoader", "neigh", "all", "local"):
            try:
                perf[k] = ctx.metrics(k)
            except Exception:
                perf[k] = None
    # per-cell flops and bytes of each proxy kernel: the estimate of the whole step and the
    # kernels that one step of it launches (ADER, local integral, neighbour flux)
    launched = {"all": ("ader", "localwoader", "neigh"), "local": ("ader", "localwoader"), "neigh": ("neigh",),
                "ader": ("ader",), "localwoader": ("localwoader",)}
    flop = kbytes = ebytes = 0.0
    for k in cfg.kernels:
        if perf.get(k):
            flop += perf[k]["nonzero_flop"]
            ebytes += perf[k]["bytes"]
        for part in launched.get(k, ()):
            if perf.get(part):
                kbytes += perf[part]["bytes"]
    if cfg.mechanisms:  # the per-kernel counts above are the elastic kernels'
        flop = kbytes = 0.0
        ebytes = bytes_per_cell(cfg.order, cfg.mechanisms) * len(cfg.kernels)
    elif ebytes == 0.0:  # fault kernels: the step model of the elastic update
        ebytes = bytes_per_cell(cfg.order) * len(cfg.kernels)
    work = n * cfg.timesteps
    secs = total_ms / 1e3 if total_ms > 0 else wall
    try:
        from .lib import device_clock_khz
        cycles = secs * device_clock_khz(cfg.device) * 1e3
    except Exception:
        cycles = 0.0
    gflop = flop * work / 1e9
    gib, kgib = ebytes * work / 2 ** 30, kbytes * work / 2 ** 30
    per_cycle = (lambda v: v / cycles) if cycles > 0 else (lambda v: 0.0)
    return ProxyOutput(time=secs, cycles=cycles, actualNonZeroGFlop=gflop, actualHardwareGFlop=gflop, gib=gib,
                       kernelGib=kgib, nonZeroFlopPerCycle=per_cycle(gflop * 1e9),
                       hardwareFlopPerCycle=per_cycle(gflop * 1e9), bytesPerCycle=per_cycle(ebytes * work),
                       kernelBytesPerCycle=per_cycle(kbytes * work), nonZeroGFlops=gflop / secs,
                       hardwareGFlops=gflop / secs, gibPerSecond=gib / secs, kernelGibPerSecond=kgib / secs,
                       cellUpdatesPerSecond=work / secs)


def write_output(out: ProxyOutput, name: str, fmt: str = "plain", stream=sys.stdout):
    """Plain or JSON summary with the fields and keys of src/Proxy/Common.cpp:87-154, plus the
    cell-update rate of this project's metric."""
    if fmt == "json":
        stream.write(json.dumps({"name": name, "time": out.time, "cycles": out.cycles,
                                 "gflop-libxsmm": out.libxsmmNumTotalGFlop, "gflop-pspamm": out.pspammNumTotalGFlop,
                                 "gflop-nz": out.actualNonZeroGFlop, "gflop-hw": out.actualHardwareGFlop,
                                 "gib": out.gib, "gib-kernel": out.kernelGib,
                                 "gflopcycle-nz": out.nonZeroFlopPerCycle, "gflopcycle-hw": out.hardwareFlopPerCycle,
                                 "gibcycle": out.bytesPerCycle, "gibcycle-kernel": out.kernelBytesPerCycle,
                                 "gflops-nz": out.nonZeroGFlops, "gflops-hw": out.hardwareGFlops,
                                 "gibs": out.gibPerSecond, "gibs-kernel": out.kernelGibPerSecond,
                                 "cell-updates-per-s": out.cellUpdatesPerSecond}) + "\n")
        return
    rows = (("seissol proxy mode", name), ("time for seissol proxy", out.time), ("cycles", out.cycles), None,
            ("GFLOP (libxsmm)", out.libxsmmNumTotalGFlop), ("GFLOP (pspamm)", out.pspammNumTotalGFlop),
            ("GFLOP (libxsmm + pspamm)", out.libxsmmAndpspammNumTotalGFlop),
            ("GFLOP (non-zero) for seissol proxy", out.actualNonZeroGFlop),
            ("GFLOP (hardware) for seissol proxy", out.actualHardwareGFlop),
            ("GiB (estimate) for seissol proxy", out.gib), ("GiB (kernels) for seissol proxy", out.kernelGib), None,
            ("FLOPS/cycle (non-zero)", out.nonZeroFlopPerCycle), ("FLOPS/cycle (hardware)", out.hardwareFlopPerCycle),
            ("Bytes/cycle (estimate)", out.bytesPerCycle), ("Bytes/cycle (kernel)", out.kernelBytesPerCycle), None,
            ("GFLOPS (non-zero) for seissol proxy", out.nonZeroGFlops),
            ("GFLOPS (hardware) for seissol proxy", out.hardwareGFlops),
            ("GiB/s (estimate) for seissol proxy", out.gibPerSecond),
            ("GiB/s (kernel) for seissol proxy", out.kernelGibPerSecond), ("cell updates/s", out.cellUpdatesPerSecond))
    stream.write("=================================================\n")
    stream.write("===            PERFORMANCE SUMMARY            ===\n")
    stream.write("=================================================\n")
    for row in rows:
        stream.write("\n" if row is None else f"{row[0]:<36}: {row[1]}\n")
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
    ap.add_argument("--plasticity", action="store_true", help="off-fault plasticity on every cell (elastic)")
    ap.add_argument("--mechanisms", type=int, choices=(0, 3), default=0,
                    help="3: viscoelastic equations with three relaxation mechanisms (orders 4 and 5)")
    a = ap.parse_args(argv)
    kernels = tuple(Aux.str_to_kernel(a.kernel))
    out = run_proxy(ProxyConfig(cells=a.cells, timesteps=a.timesteps, kernels=kernels, order=a.order,
                                precision={"fp32": 0, "f16x3": 1}[a.precision], mechanisms=a.mechanisms,
                                plasticity=a.plasticity))
    write_output(out, a.kernel, a.format)
    return 0


if __name__ == "__main__":
    sys.exit(main())
