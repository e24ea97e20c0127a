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


@pytest.mark.parametrize("precision", [32, 64])
def test_uploaded_members_bit_identical_to_alone(axs, precision):
    """Members given a full state by upload (whose first step, a pure drift,
    is formed by the upload) evolve as the same states uploaded to lattices
    run alone, before and after the ensemble has been tuned."""
    specs = [(32, 1.0), (48, 2.0), (64, 0.7)]
    plist = [params(axs, 3, N, precision, lambda_=lam, T_initial=0.0, prs=1) for N, lam in specs]
    dt = np.float32 if precision == 32 else np.float64
    rng = np.random.default_rng(21)
    states = [[rng.standard_normal((N, N, N)).astype(dt) for _ in range(4)] for N, _ in specs]
    with axs.Ensemble(plist) as E:
        got = []
        for rnd in range(2):   # the first evolve tunes the ensemble, the second finds it tuned
            times = [m.time for m in E.members]   # an upload keeps a lattice's time
            for m, f in zip(E.members, states):
                m.upload(*f, dtype=dt)
            E.evolve(9)
            got.append([(t, m.download(dtype=dt)) for t, m in zip(times, E.members)])
    for rnd in range(2):
        for p, f, (t, g) in zip(plist, states, got[rnd]):
            with axs.Lattice(p) as L:
                L.set_time(*t)
                L.upload(*f, dtype=dt)
                L.evolve(9)
                ref = L.download(dtype=dt)
            for q in range(4):
                assert np.array_equal(g[q], ref[q]), (rnd, q)


@pytest.mark.parametrize("force", ["1,10,32", "1,13,64", "1,12,128", "1,28,128", "1,31,128", "1,39,64"])
def test_two_step_members_bit_identical_to_one_step_alone(axs, force, monkeypatch):
    """An ensemble on a two-step variant (halo depth 2, momentum out of place)
    matches each member run alone with the one-step kernel, over even and odd
    intervals."""
    specs = [(160, 1.0, 31), (64, 0.7, 32), (96, 2.5, 33), (32, 0.5, 34)]
    plist = [params(axs, 3, N, 32, lambda_=lam, T_initial=0.0, prs=1) for N, lam, _ in specs]
    monkeypatch.setenv("AXS_FORCE_CONFIG", force)
    with axs.Ensemble(plist) as E:
        for m, (_, _, seed) in zip(E.members, specs):
            m.init_flat(seed, 1.0)
        for n in (1, 4, 3, 1, 6):
            E.evolve(n)
        assert "two steps per pass" in E.describe(), E.describe()
        res_e = [(m.download(dtype=np.float32), m.time) for m in E.members]
    monkeypatch.setenv("AXS_FORCE_CONFIG", "0,0,64")
    for (N, lam, seed), p, (fe, te) in zip(specs, plist, res_e):
        with axs.Lattice(p) as L:
            L.init_flat(seed, 1.0)
            L.evolve(15)
            f = L.download(dtype=np.float32)
            assert L.time == te
        for q in range(4):
            assert np.array_equal(f[q], fe[q]), (N, q)


def test_ensemble_rejects_mixed_precision(axs):
    with pytest.raises(axs.AxsError):
        axs.Ensemble([params(axs, 3, 32, 32), params(axs, 3, 32, 64)])


@pytest.mark.parametrize("precision", [32, 64])
def test_batched_analysis_equals_per_member_calls(axs, precision):
    """axs_ensemble_find_strings / axs_ensemble_axion_spectrum (every member's
    kernels back to back, one synchronisation) give the per-member calls'
    bits, on the first call of a binning and on later ones."""
    specs = [(64, 1.0, 41), (32, 0.6, 42), (48, 2.0, 43), (64, 3.0, 44)]
    plist = [params(axs, 3, N, precision, lambda_=lam, T_initial=0.0, prs=1) for N, lam, _ in specs]
    with axs.Ensemble(plist) as E:
        for m, (_, _, seed) in zip(E.members, specs):
            m.init_flat(seed, 1.0)
        E.evolve(12)
        for rep in range(2):
            npl, nco = E.find_strings()
            k, pk, cnt = E.axion_spectrum(24)
            for i, m in enumerate(E.members):
                n1, c1, _ = m.find_strings()
                assert (n1, c1) == (npl[i], nco[i])
                k1, pk1, cnt1 = m.axion_spectrum(24)
                assert np.array_equal(k1, k[i]) and np.array_equal(pk1, pk[i]) and np.array_equal(cnt1, cnt[i])
            E.evolve(2)
