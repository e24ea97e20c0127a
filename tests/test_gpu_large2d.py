"""Large 2D lattices (the reference runs 2D string networks far above the 3D
sizes): the spectrum binner splits rows into segments and bins into passes
once one block's shared memory cannot hold them, and forms |n| in double
where |n|^2 >= 2^24. Spectra against the oracle; steps FP32 against FP64."""
import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,precision", [(4096, 64), (4096, 32), (8192, 32)])
def test_large_2d_powerspec_matches_oracle(axs, oracle, N, precision):
    p = params(axs, 2, N, precision, T_initial=0.0)
    with axs.Lattice(p) as L:
        L.init_flat(7, 1.0)
        L.evolve(3)
        g = L.download()
        pk, ks, cnt = L.powerspec(1)
        pk2, ks2, cnt2 = L.powerspec(1)   # the binning's |n| sums and counts reused: same bits
    assert np.array_equal(pk, pk2, equal_nan=True) and np.array_equal(ks, ks2, equal_nan=True)
    assert np.array_equal(cnt, cnt2)
    pko, kso, cnto = oracle.powerspec(orc(params(axs, 2, N, 64)), g[1])
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= (1e-11 if precision == 64 else 1e-5)
    assert rel(ks[ok], kso[ok]) <= 1e-11


def test_large_2d_step_fp32_against_fp64(axs):
    N = 16384
    p64, p32 = params(axs, 2, N, 64, T_initial=0.0), params(axs, 2, N, 32, T_initial=0.0)
    with axs.Lattice(p64) as A:
        A.init_flat(9, 1.0)
        f = A.download()
        A.evolve(10)
        ga = A.download()
        n_a, _, _ = A.find_strings()
        ka, pka, ca = A.axion_spectrum(64)
    with axs.Lattice(p32) as B:
        B.upload(*f)
        B.evolve(10)
        gb = B.download()
        n_b, _, _ = B.find_strings()
        kb, pkb, cb = B.axion_spectrum(64)
    for q in range(4):
        assert np.isfinite(gb[q]).all()
        assert rel(gb[q], ga[q]) <= 1e-5, (q, rel(gb[q], ga[q]))
    assert np.array_equal(ca, cb)
    ok = ca > 0
    assert rel(pkb[ok], pka[ok]) <= 1e-4
    assert abs(n_a - n_b) <= max(2, n_a // 1000)
