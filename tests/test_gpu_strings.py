"""String finder: bit-exact to cores2/cores3 (src/common/string_finding.cpp)
on a given theta; theta = atan2(phi1, phi2) computed on the device otherwise."""
import os

import numpy as np
import pytest

from gpu_util import orc, params
from strings_util import accept_value, near_threshold_theta

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


def test_xi_matches_reference_float_formula(axs, oracle):
    for nd, N in [(2, 512), (3, 256)]:
        p = params(axs, nd, N, 64)
        for tau, n, c in [(1.0, 100, 90), (37.3, 12345, 12000), (128.6, 5, 5)]:
            assert axs.xi(p, n, c, tau) == oracle.xi(orc(p), n, c, tau)
