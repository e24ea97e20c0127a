"""The smallest lattices the reference accepts (N even, N >= 4, N > 2 x the
stencil radius): steps, strings and spectra against the oracle, so the tile
and halo logic of every kernel holds when one tile wraps onto itself."""
import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nd,N", [(2, 4), (2, 6), (3, 4), (3, 6), (3, 8)])
@pytest.mark.parametrize("precision", [64, 32])
def test_smallest_lattices(axs, oracle, nd, N, precision):
    p = params(axs, nd, N, precision)
    op = orc(params(axs, nd, N, 64))
    f = oracle.init_thermal(op, 5)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(1)
        L.evolve(6)   # a graph-replayed interval after a single step
        g = L.download()
        tau, steps = L.time
        n_g, _, mask_g = L.find_strings(want_mask=True)
        pk, ks, cnt = L.powerspec(1)
        if nd == 3:
            k, apk, acnt = L.axion_spectrum(4)
    o = oracle.evolve(op, *f, 7)
    tol = 1e-12 if precision == 64 else 1e-5
    for q in range(4):
        assert rel(g[q], o[q]) <= tol, (q, rel(g[q], o[q]))
    assert steps == 7 and tau == o[4]
    if precision == 64:
        # decisions from the device's own field; FP64 atan2 may differ from the
        # host's in the last ulp, which could move a cell sitting on the threshold
        n_o, mask_o = oracle.cores(op, np.arctan2(g[0], g[1]))
        assert int(np.count_nonzero(mask_g != mask_o)) <= 1
        pko, kso, cnto = oracle.powerspec(op, g[1])
        assert np.array_equal(cnt, cnto)
        ok = cnto > 0
        assert rel(pk[ok], pko[ok]) <= 1e-11
        if nd == 3:
            ko, apko, acnto = oracle.axion_spectrum(op, *g, tau, 4)
            assert np.array_equal(acnt, acnto)
            ok = acnto > 0
            assert rel(apk[ok], apko[ok]) <= 1e-10
