"""Initial conditions: GPU (Philox + Box-Muller in k-space, cuFFT Z2Z
inverse) against the oracle restatement of gaussian_thermal
(src/common/init.cpp:33-200) and of the flat k_cut field. FP64, 1e-12."""
import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,N", [(2, 64), (3, 32), (3, 48)])
def test_thermal_init_matches_oracle(axs, oracle, nd, N):
    p = params(axs, nd, N, 64, T_initial=4.0, lambda_=1.0)
    with axs.Lattice(p) as L:
        L.init_thermal(17)
        g = L.download()
        assert L.time == (1.0, 0)
    o = oracle.init_thermal(orc(p), 17)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-12, (q, rel(g[q], o[q]))


@pytest.mark.parametrize("nd,N,kcut", [(2, 128, 1.0), (3, 32, 1.0), (3, 64, 2.0)])
def test_flat_init_matches_oracle(axs, oracle, nd, N, kcut):
    p = params(axs, nd, N, 64)
    with axs.Lattice(p) as L:
        L.init_flat(23, kcut)
        g = L.download()
    o = oracle.init_flat(orc(p), 23, kcut)
    for q in range(2):
        assert rel(g[q], o[q]) <= 1e-12
    assert np.all(g[2] == 0) and np.all(g[3] == 0)
    assert abs(np.mean(g[0] ** 2 + g[1] ** 2) - 1.0) < 1e-12


def test_fp32_lattice_starts_from_rounded_fp64_field(axs):
    p64 = params(axs, 3, 32, 64)
    p32 = params(axs, 3, 32, 32)
    with axs.Lattice(p64) as A, axs.Lattice(p32) as B:
        A.init_flat(5, 1.0)
        B.init_flat(5, 1.0)
        a = A.download()
        b = B.download(dtype=np.float32)
    for q in range(2):
        assert np.array_equal(a[q].astype(np.float32), b[q])
