"""The proxy's kernel-name helpers and output (the reference's Aux, src/Proxy/Common.cpp and
app/Proxy/Bindings.cpp): names round-trip, unknown names raise, the plain and JSON outputs carry
the reference's fields and keys.  Host only."""
import io
import json

import pytest

from seissol_gb300.proxy import Aux, ProxyOutput, write_output


def test_kernel_names_round_trip():
    allowed = Aux.get_allowed_kernels()
    assert set(allowed) == {"all", "local", "neigh", "ader", "localwoader", "neigh_dr", "godunov_dr", "all_dr"}
    assert Aux.str_to_kernel(" all, neigh ,ader") == ["all", "neigh", "ader"]
    assert Aux.kernel_to_string(["all_dr", "local"]) == "all_dr,local"
    with pytest.raises(ValueError):
        Aux.str_to_kernel("all,bogus")
    with pytest.raises(ValueError):
        Aux.kernel_to_string(["bogus"])


def test_output_fields():
    out = ProxyOutput(time=2.0, cycles=4e9, actualNonZeroGFlop=10.0, gib=3.0, kernelGib=5.0, nonZeroGFlops=5.0,
                      gibPerSecond=1.5, kernelGibPerSecond=2.5, cellUpdatesPerSecond=7.0)
    assert out.actual_non_zero_gflop == 10.0 and out.gib_per_second == 1.5
    s = io.StringIO()
    write_output(out, "all", "json", s)
    d = json.loads(s.getvalue())
    for key in ("name", "time", "cycles", "gflop-libxsmm", "gflop-pspamm", "gflop-nz", "gflop-hw", "gib", "gib-kernel",
                "gflopcycle-nz", "gflopcycle-hw", "gibcycle", "gibcycle-kernel", "gflops-nz", "gflops-hw", "gibs",
                "gibs-kernel"):
        assert key in d, key
    assert d["gib-kernel"] == 5.0 and d["cycles"] == 4e9
    s = io.StringIO()
    Aux.write_output(s, out, "all")
    text = s.getvalue()
    for label in ("seissol proxy mode", "cycles", "GiB (kernels) for seissol proxy", "Bytes/cycle (kernel)",
                  "GiB/s (kernel) for seissol proxy"):
        assert label in text, label
