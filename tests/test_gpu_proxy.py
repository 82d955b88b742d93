"""The seissol-proxy equivalent (seissol_gb300.proxy) over the C ABI: every kernel name of the
reference proxy runs and reports positive throughput; the *_dr kernels run on a planar fault."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernels,order,precision", [(("all",), 6, 0), (("local", "neigh", "ader", "localwoader"), 5, 0),
                                                     (("all",), 4, 1), (("all_dr", "neigh_dr", "godunov_dr"), 4, 0)])
def test_proxy_kernels(built_lib, kernels, order, precision):
    from seissol_gb300.proxy import ProxyConfig, run_proxy
    out = run_proxy(ProxyConfig(cells=4000, timesteps=2, kernels=kernels, order=order, precision=precision))
    assert out.time > 0 and out.cellUpdatesPerSecond > 0 and out.cycles > 0
    if "all" in kernels or "local" in kernels:
        assert out.nonZeroGFlops > 0 and out.nonZeroFlopPerCycle > 0
        # the launched kernels move more than the step's compulsory estimate (I is written and re-read)
        assert out.kernelGib > out.gib > 0


def test_proxy_rejects_unknown_kernel(built_lib):
    from seissol_gb300.proxy import ProxyConfig, run_proxy
    with pytest.raises(ValueError):
        run_proxy(ProxyConfig(cells=100, timesteps=1, kernels=("bogus",)))
