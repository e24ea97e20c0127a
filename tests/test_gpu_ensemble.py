"""Batched ensembles: one persistent launch per step over uneven lattices;
every member is bit-identical to the same lattice run alone (fields, string
counts, spectra)."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [32, 64])
def test_members_bit_identical_to_alone(axs, precision):
    specs = [(64, 1.0, 11), (32, 0.7, 12), (48, 2.5, 13), (96, 3.9, 14), (32, 0.5, 15)]
    plist = [params(axs, 3, N, precision, lambda_=lam, T_initial=0.0, prs=1) for N, lam, _ in specs]
    with axs.Ensemble(plist) as E:
        for m, (_, _, seed) in zip(E.members, specs):
            m.init_flat(seed, 1.0)
        E.evolve(1)
        E.evolve(12)
        E.evolve(12)
        res_e = []
        for m in E.members:
            f = m.download(dtype=np.float64)
            n, c, _ = m.find_strings()
            pk = m.axion_spectrum(32)
            res_e.append((f, n, pk))
    for (N, lam, seed), p, (fe, ne, pke) in zip(specs, plist, res_e):
        with axs.Lattice(p) as L:
            L.init_flat(seed, 1.0)
            L.evolve(25)
            f = L.download(dtype=np.float64)
            n, c, _ = L.find_strings()
            pk = L.axion_spectrum(32)
        for q in range(4):
            assert np.array_equal(f[q], fe[q]), (N, q)
        assert n == ne
        for a, b in zip(pk, pke):
            assert np.array_equal(a, b)


def test_ensemble_rejects_mixed_precision(axs):
    with pytest.raises(axs.AxsError):
        axs.Ensemble([params(axs, 3, 32, 32), params(axs, 3, 32, 64)])
