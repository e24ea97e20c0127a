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


@pytest.mark.parametrize("nd,N", [(2, 64), (2, 48), (3, 32), (3, 24)])
def test_spectral_laplacian_matches_oracle(axs, oracle, nd, N):
    """laplacian = 1: compute_laplacian_fft (s_integrate.cpp:179-296) through
    cuFFT, against the oracle (pinned to the reference's own function), FP64
    within 1e-12 of the largest value; both components."""
    from gpu_util import orc
    p = params(axs, nd, N, 64, space_step=0.7, laplacian=1)
    rng = np.random.default_rng(nd * 7 + N)
    f1, f2 = rng.standard_normal((N,) * nd), rng.standard_normal((N,) * nd)
    with axs.Lattice(p) as L:
        L.upload(f1, f2, np.zeros_like(f1), np.zeros_like(f1))
        g1, g2 = L.laplacian(0), L.laplacian(1)
    o1, o2 = oracle.laplacian(orc(p), f1), oracle.laplacian(orc(p), f2)
    assert np.abs(g1 - o1).max() <= 1e-12 * np.abs(o1).max()
    assert np.abs(g2 - o2).max() <= 1e-12 * np.abs(o2).max()


@pytest.mark.parametrize("precision,tol", [(64, 1e-11), (32, 5e-5)])   # FP32: a transform pair of 64^3
def test_spectral_laplacian_plane_wave(axs, precision, tol):
    """The spectral Laplacian of a lattice plane wave is -k^2 times it."""
    N, dx = 64, 0.5
    p = params(axs, 3, N, precision, space_step=dx, laplacian=1)
    I, J, K = np.indices((N, N, N))
    n = (3, 1, 2)
    f = np.cos(2 * np.pi * (n[0] * I + n[1] * J + n[2] * K) / N + 0.3)
    k2 = sum((2 * np.pi * q / (N * dx)) ** 2 for q in n)
    with axs.Lattice(p) as L:
        L.upload(f, np.zeros_like(f), np.zeros_like(f), np.zeros_like(f))
        lap = L.laplacian(0)
    assert np.abs(lap + k2 * f).max() <= tol * k2
