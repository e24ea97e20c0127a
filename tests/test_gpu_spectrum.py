"""Spectra: output_powerspec (src/common/pk_estimation.cpp:37-214) and the
axion kinetic-energy spectrum, against the oracle. FP64 bins within 1e-11
relative; FP32 fields within 1e-5."""
import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,N", [(2, 64), (2, 96), (3, 32), (3, 48)])
@pytest.mark.parametrize("field", [1, 0, 3])
def test_powerspec_matches_oracle(axs, oracle, nd, N, field):
    p = params(axs, nd, N, 64)
    op = orc(p)
    f = oracle.init_thermal(op, 8)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(5)
        g = L.download()
        pk, ks, cnt = L.powerspec(field)
    pko, kso, cnto = oracle.powerspec(op, g[field])
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-11
    assert rel(ks[ok], kso[ok]) <= 1e-11
    assert np.all(np.isnan(pk[~ok])) and np.all(np.isnan(ks[~ok]))


def test_powerspec_fp32(axs, oracle):
    p = params(axs, 3, 32, 32)
    op = orc(p)
    f = oracle.init_thermal(op, 8)
    with axs.Lattice(p) as L:
        L.upload(*f)
        pk, ks, cnt = L.powerspec(1)
        g = L.download()
    pko, kso, cnto = oracle.powerspec(op, g[1])
    ok = cnto > 0
    assert np.array_equal(cnt, cnto)
    assert rel(pk[ok], pko[ok]) <= 1e-5


@pytest.mark.parametrize("nd,N,nbins,stencil", [(3, 32, 16, 0), (3, 48, 128, 0), (2, 64, 32, 0),
                                                (3, 40, 32, 1), (3, 24, 16, 2), (3, 36, 24, 3), (2, 48, 16, 3)])
def test_axion_spectrum_matches_oracle(axs, oracle, nd, N, nbins, stencil):
    """3D finite-difference stencils of every radius form pi_n in the z-column
    march; 2D forms it in scratch first."""
    p = params(axs, nd, N, 64, T_initial=0.0, stencil_setting=stencil)
    op = orc(p)
    f = oracle.init_flat(op, 2, 2.0)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(20)
        g = L.download()
        tau, _ = L.time
        k, pk, cnt = L.axion_spectrum(nbins)
    ko, pko, cnto = oracle.axion_spectrum(op, *g, tau, nbins)
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-10
    assert rel(k[ok], ko[ok]) <= 1e-12


@pytest.mark.parametrize("N,nbins,stencil", [(40, 24, 0), (32, 16, 0), (40, 24, 3)])
def test_axion_spectrum_fresh_state(axs, oracle, N, nbins, stencil):
    """Right after an upload the momentum is pi_0 itself (no stencil term)."""
    p = params(axs, 3, N, 64, T_initial=0.0, stencil_setting=stencil)
    op = orc(p)
    f = oracle.init_flat(op, 5, 2.0)
    with axs.Lattice(p) as L:
        L.upload(*f)
        tau, _ = L.time
        k, pk, cnt = L.axion_spectrum(nbins)
    ko, pko, cnto = oracle.axion_spectrum(op, *f, tau, nbins)
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-10
    assert rel(k[ok], ko[ok]) <= 1e-12


@pytest.mark.parametrize("stencil", [0, 2])
def test_axion_spectrum_fp32(axs, oracle, stencil):
    """FP32 fields: the spectrum of the downloaded (FP32) state within 1e-4."""
    p = params(axs, 3, 48, 32, T_initial=0.0, stencil_setting=stencil)
    op = orc(p)
    f = oracle.init_flat(op, 6, 2.0)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(9)
        g = L.download()
        tau, _ = L.time
        k, pk, cnt = L.axion_spectrum(32)
    ko, pko, cnto = oracle.axion_spectrum(op, *g, tau, 32)
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-4
    assert rel(k[ok], ko[ok]) <= 1e-6


@pytest.mark.parametrize("nd,N", [(3, 48), (2, 64)])
def test_repeated_spectra_reuse_bin_geometry(axs, oracle, nd, N):
    """A binning's |n| sums and counts come from its first call and are reused
    by later calls, which sum the power alone: repeated calls on one state,
    with other binnings in between, give the same bits, and a later state
    still matches the oracle."""
    p = params(axs, nd, N, 64, T_initial=0.0)
    op = orc(p)
    f = oracle.init_flat(op, 4, 2.0)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(6)
        a1 = L.axion_spectrum(32)
        s1 = L.powerspec(1)
        a2 = L.axion_spectrum(20)
        s2 = L.powerspec(1)
        a3 = L.axion_spectrum(32)
        for x, y in zip(a1, a3):
            assert np.array_equal(x, y)
        for x, y in zip(s1, s2):
            assert np.array_equal(x, y, equal_nan=True)
        L.evolve(5)
        g = L.download()
        tau, _ = L.time
        k, pk, cnt = L.axion_spectrum(20)
        ps, ks, cs = L.powerspec(1)
    ko, pko, cnto = oracle.axion_spectrum(op, *g, tau, 20)
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-10
    assert rel(k[ok], ko[ok]) <= 1e-12
    pso, kso, cso = oracle.powerspec(op, g[1])
    assert np.array_equal(cs, cso)
    ok = cso > 0
    assert rel(ps[ok], pso[ok]) <= 1e-11
    assert rel(ks[ok], kso[ok]) <= 1e-11
