"""The reference's known-answer Laplacian tests (src/tests/laplacian.cpp:13-87,
src/tests/fdm_matrix.cpp:109-244) through the device stencil: zeros give
zero; sin/cos waves with L = N/2, dx = 1 match -(pi/L)^2 f within 1e-5."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,N", [(2, 128), (2, 256), (3, 128), (3, 256)])
@pytest.mark.parametrize("precision", [64, 32])
def test_wave_known_answer(axs, nd, N, precision):
    p = params(axs, nd, N, precision, space_step=1.0)
    L_ = N / 2.0
    i = np.arange(N)
    if nd == 2:
        jj, ii = np.meshgrid(i, i, indexing="ij")   # a[j, i]
        f = np.sin(np.pi / L_ * ii) + np.cos(np.pi / L_ * jj)
    else:
        I, J, K = np.meshgrid(i, i, i, indexing="ij")
        f = np.sin(np.pi / L_ * I) + np.cos(np.pi / L_ * J) + np.sin(np.pi / L_ * K)
    with axs.Lattice(p) as L:
        L.upload(f, np.zeros_like(f), np.zeros_like(f), np.zeros_like(f))
        lap = L.laplacian(0)
        zero = L.laplacian(1)
    assert np.abs(lap - (-(np.pi / L_) ** 2) * f).max() <= 1e-5
    assert np.abs(zero).max() <= 1e-30
