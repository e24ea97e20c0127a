"""Background means (s_run.cpp:135-150), energies and the finite check."""
import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-6)])
@pytest.mark.parametrize("nd,N,stencil,steps,prs,lap", [
    (2, 64, 0, 15, 1, 0), (3, 32, 0, 15, 1, 0),
    (3, 20, 0, 15, 1, 0),    # columns past the edge of the 32 x 8 blocks
    (3, 36, 0, 9, 0, 0),
    (3, 32, 0, 0, 1, 0),     # a fresh state: pih holds pi_0
    (3, 24, 1, 15, 1, 0),    # radius 2..4: the z-column march of that radius
    (3, 24, 2, 15, 1, 0),
    (3, 20, 3, 9, 0, 0),     # radius 4, columns past the edge of the blocks
    (3, 24, 3, 0, 1, 0),     # radius 4, fresh
    (3, 16, 0, 6, 1, 1),     # spectral Laplacian
    (2, 48, 3, 12, 1, 0),    # radius 4 in 2D
])
def test_background_and_energies(axs, oracle, precision, tol, nd, N, stencil, steps, prs, lap):
    """The device's background means take the mean of pi_n without the
    Laplacian part of the half kick (it sums to zero over the periodic
    lattice); the oracle averages the per-site pi_n that download() forms with
    the full stencil, so these cases also check that cancellation for every
    stencil and the spectral operator."""
    p = params(axs, nd, N, precision, T_initial=0.0, stencil_setting=stencil, prs=prs, laplacian=lap)
    op = orc(p)
    with axs.Lattice(p) as L:
        L.init_flat(6, 1.0)
        if steps:
            L.evolve(steps)
        g = L.download()
        tau, _ = L.time
        bg = L.background()
        en = L.energies()
    bo = oracle.background(op, *g)
    eo = oracle.energies(op, *g, tau)
    for q in range(6):
        assert abs(bg[q] - bo[q]) <= tol * max(1.0, abs(bo[q])), (q, bg[q], bo[q])
    for q in range(3):
        assert abs(en[q] - eo[q]) <= tol * max(1e-3, abs(eo[q])) * 10, (q, en[q], eo[q])


def test_finite_check_flags_seeded_nan(axs):
    p = params(axs, 3, 32, 64)
    with axs.Lattice(p) as L:
        L.init_flat(1, 1.0)
        assert L.check_finite()
        f = list(L.download())
        f[2][3, 4, 5] = np.nan
        L.upload(*f)
        assert not L.check_finite()


def test_background_angle_and_modulus_edge_cases(axs):
    """FP64 means of |theta| = |atan2(phi1, phi2)| and |phi| over sites that
    the table rotation serves and sites it hands to the library (zeros, values
    outside float range, the branch cut at theta = +-pi), against numpy, on a
    fresh state (pi_n is the uploaded pi)."""
    N = 4
    p = params(axs, 3, N, 64)
    rng = np.random.default_rng(5)
    p1 = rng.standard_normal(N ** 3)
    p2 = rng.standard_normal(N ** 3)
    special = [(0.0, 0.0), (0.0, -1.0), (-0.0, -1.0), (1e-13, -1.0), (-1e-13, -1.0), (1.0, 0.0), (-1.0, 0.0),
               (1e100, 3e100), (-2e-200, 1e-200), (3e-40, -5e-40), (1e-300, -2.0), (2.5, -1e-17)]
    for i, (a, b) in enumerate(special):
        p1[i], p2[i] = a, b
    z = np.zeros(N ** 3)
    with axs.Lattice(p) as L:
        L.upload(p1.reshape(N, N, N), p2.reshape(N, N, N), z.reshape(N, N, N), z.reshape(N, N, N))
        bg = L.background()
    th = np.mean(np.abs(np.arctan2(p1, p2)))
    ph = np.mean(np.sqrt(p1 * p1 + p2 * p2))
    assert abs(bg[4] - th) <= 1e-15 * th, (bg[4], th)
    assert abs(bg[5] - ph) <= 1e-15 * ph, (bg[5], ph)
