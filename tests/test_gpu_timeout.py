"""Failure path without a GPU fault: a step whose TMA loads never complete
their mbarrier phase (injected from the host) runs its bounded waits out,
returns, and is reported as AXS_ERR_TIMEOUT; the context stays usable."""
import os
import time

import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("force", ["1,7,32", "1,0,32"])   # producer-warp kernel, CTA-barrier kernel
def test_wait_timeout_is_reported_and_context_survives(axs, oracle, force):
    os.environ["AXS_FORCE_CONFIG"] = force
    try:
        with axs.Lattice(params(axs, 3, 64, 32)) as L:
            L.init_flat(1, 1.0)
            L.evolve(1)                       # the initial drift (no device-side waits)
            L.inject_wait_timeout()
            t0 = time.time()
            with pytest.raises(axs.AxsError) as e:
                L.evolve_timed(1)
            assert e.value.code == axs.ERR_TIMEOUT
            assert time.time() - t0 < 60
    finally:
        del os.environ["AXS_FORCE_CONFIG"]
    # the context still works: a new lattice steps and matches the oracle
    p = params(axs, 3, 32, 64)
    f = oracle.init_thermal(orc(p), 4)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(5)
        g = L.download()
    o = oracle.evolve(orc(p), *f, 5)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-12


def test_injection_needs_the_tma_kernel(axs):
    os.environ["AXS_FORCE_CONFIG"] = "0,0,64"
    try:
        with axs.Lattice(params(axs, 3, 32, 64)) as L:
            with pytest.raises(axs.AxsError) as e:
                L.inject_wait_timeout()
            assert e.value.code == axs.ERR_STATE
    finally:
        del os.environ["AXS_FORCE_CONFIG"]
