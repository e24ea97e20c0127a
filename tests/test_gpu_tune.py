"""The autotuner times its candidates with dt = 0 steps on the lattice's own
buffers: a finite state comes back bit-identical, and a state holding an
Inf is not timed on (0 * Inf would turn it into NaN). Each test uses a shape
no other test tunes, so the trials run (tuned shapes are cached per process)."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


def _state(N, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((N, N, N)).astype(np.float32) for _ in range(4)]


def test_tuning_leaves_finite_state_bit_identical(axs):
    p = params(axs, 3, 112, 32)
    f = _state(112, 1)
    with axs.Lattice(p) as L:
        L.upload(*f, dtype=np.float32)
        L.autotune()
        assert "z-march" in L.describe(), L.describe()
        g = L.download(dtype=np.float32)
        tau, steps = L.time
    assert steps == 0 and tau == 1.0
    for q in range(4):
        assert np.array_equal(g[q], f[q]), q


def test_tuning_skips_non_finite_state(axs):
    p = params(axs, 3, 80, 32)
    f = _state(80, 2)
    f[2][5, 6, 7] = np.inf
    with axs.Lattice(p) as L:
        L.upload(*f, dtype=np.float32)
        assert not L.check_finite()
        L.autotune()
        g = L.download(dtype=np.float32)
    assert np.isposinf(g[2][5, 6, 7])
    for q in range(4):
        assert np.array_equal(g[q], f[q]), q
