"""String finder: bit-exact to cores2/cores3 (src/common/string_finding.cpp)
on a given theta; theta = atan2(phi1, phi2) computed on the device otherwise."""
import os

import numpy as np
import pytest

from gpu_util import orc, params
from strings_util import accept_value, cell_sums3, near_threshold_theta

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("nd,N,thr", [(2, 64, 1), (2, 96, 30), (3, 24, 1), (3, 32, 0)])
def test_bit_exact_on_given_theta(axs, oracle, nd, N, thr):
    p = params(axs, nd, N, 64, thr=thr)
    accept = accept_value(thr)
    rng = np.random.default_rng(N + thr)
    for theta in (rng.uniform(-np.pi, np.pi, (N,) * nd), near_threshold_theta(rng, nd, N, accept)):
        n_o, mask_o = oracle.cores(orc(p), theta)
        with axs.Lattice(p) as L:
            n_g, cores_g, mask_g = L.find_strings(theta=theta, want_mask=True)
            pos = L.string_positions()
        assert n_g == n_o
        assert np.array_equal(mask_g, mask_o)
        idx = np.flatnonzero(mask_o.reshape(-1))
        if nd == 2:
            assert np.array_equal(pos[:, 0] + N * pos[:, 1], idx)
            assert cores_g == oracle.num_cores2(N, mask_o)
        else:
            assert np.array_equal((pos[:, 0] * N + pos[:, 1]) * N + pos[:, 2], idx)
            assert cores_g == n_g


def test_golden_theta_snapshots(axs):
    """Masks produced by the reference's own cores2/cores3 (fixtures)."""
    files = sorted(f for f in os.listdir(GOLD) if f.startswith("strings_"))
    assert files
    for f in files:
        z = np.load(os.path.join(GOLD, f))
        nd, N, thr = int(z["nd"]), int(z["N"]), int(z["thr"])
        theta = z["theta"]
        mask_ref = np.unpackbits(z["mask_bits"])[: theta.size].reshape(theta.shape)
        p = params(axs, nd, N, 64, thr=thr)
        with axs.Lattice(p) as L:
            n, cores, mask = L.find_strings(theta=theta, want_mask=True)
        assert n == int(z["n"]), f
        assert np.array_equal(mask, mask_ref), f
        if nd == 2:
            assert cores == int(z["num_cores_serial"]), f


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("N", [48, 40, 72])
def test_from_field_agrees_with_host_atan2(axs, oracle, precision, N):
    """theta computed on the device from psi (tiled finder; N = 40, 72 leave
    partial tiles): compared with the oracle on numpy's atan2 of the same
    (rounded) field. atan2 implementations may differ by an ulp, so the
    mismatch count is reported and must stay tiny."""
    p = params(axs, 3, N, precision)
    with axs.Lattice(p) as L:
        L.init_flat(3, 1.0)
        L.evolve(30)
        f = L.download()
        n_g, _, mask_g = L.find_strings(want_mask=True)
    theta = np.arctan2(f[0], f[1])
    n_o, mask_o = oracle.cores(orc(p), theta)
    mism = int(np.count_nonzero(mask_g != mask_o))
    print("device-theta mismatches:", mism, "of", mask_o.size, "flagged", n_o)
    assert mism <= max(2, n_o // 100000)


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("N", [30, 36, 68])
def test_from_field_near_threshold(axs, oracle, precision, N):
    """psi = (sin theta, cos theta) for a theta with many plaquette sums at
    the threshold, so many cells fall within the float stage's margin and take
    the double replay (N = 30 also leaves rows whose length is not a multiple
    of four cells). Compared with the oracle on numpy's atan2 of the same
    stored field. FP32: the rounding of psi moves those sums ~1e-7 off the
    threshold, far more than an ulp of atan2, so the masks agree. FP64: the
    sums stay within a few ulp of it, where the device's and numpy's atan2
    may round differently; every cell that differs must be such a cell."""
    p = params(axs, 3, N, precision)
    rng = np.random.default_rng(N)
    th = near_threshold_theta(rng, 3, N, accept_value(1))
    dt = np.float32 if precision == 32 else np.float64
    with axs.Lattice(p) as L:
        L.init_flat(1, 1.0)
        f = list(L.download())
        f[0] = np.sin(th).astype(dt)
        f[1] = np.cos(th).astype(dt)
        L.upload(*f)
        g = L.download()
        n_g, _, mask_g = L.find_strings(want_mask=True)
    theta = np.arctan2(g[0].astype(np.float64), g[1].astype(np.float64))
    n_o, mask_o = oracle.cores(orc(p), theta)
    mism = int(np.count_nonzero(mask_g != mask_o))
    print("near-threshold mismatches:", mism, "of", mask_o.size, "flagged", n_o)
    assert n_o > 0 and n_g == int(np.count_nonzero(mask_g))
    if precision == 32:
        assert mism == 0
    else:
        assert mism <= 10
        n = (theta + np.pi) / (2 * np.pi)
        for z, y, x in zip(*np.nonzero(mask_g != mask_o)):
            assert np.abs(cell_sums3(n, z, y, x) - accept_value(1)).min() < 1e-12, (z, y, x)


def test_xi_matches_reference_float_formula(axs, oracle):
    for nd, N in [(2, 512), (3, 256)]:
        p = params(axs, nd, N, 64)
        for tau, n, c in [(1.0, 100, 90), (37.3, 12345, 12000), (128.6, 5, 5)]:
            assert axs.xi(p, n, c, tau) == oracle.xi(orc(p), n, c, tau)
