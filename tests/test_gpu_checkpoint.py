"""Checkpoint / resume continues bit-identically (no reference counterpart)."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [32, 64])
def test_restore_continues_bit_identically(axs, precision):
    p = params(axs, 3, 32, precision)
    with axs.Lattice(p) as A:
        A.init_flat(9, 1.0)
        A.evolve(5)
        ck = A.checkpoint()
        A.evolve(6)
        a = A.download()
        ta = A.time
    with axs.Lattice(p) as B:
        B.restore(ck)
        B.evolve(6)
        b = B.download()
        assert B.time == ta
    for q in range(4):
        assert np.array_equal(a[q], b[q])


@pytest.mark.parametrize("precision", [32, 64])
def test_checkpoint_of_an_uploaded_state(axs, precision):
    """A checkpoint right after a full upload (whose first drift the upload
    already formed) restores a fresh state that continues as the original."""
    N = 32
    p = params(axs, 3, N, precision)
    dt = np.float32 if precision == 32 else np.float64
    rng = np.random.default_rng(17)
    f = [rng.standard_normal((N, N, N)).astype(dt) for _ in range(4)]
    with axs.Lattice(p) as A:
        A.init_flat(9, 1.0)
        A.evolve(2)   # tuned, so the next evolve keeps the drift the upload forms
        A.upload(*f, dtype=dt)
        ck = A.checkpoint()
        A.evolve(7)
        a = A.download(dtype=dt)
        ta = A.time
    with axs.Lattice(p) as B:
        B.restore(ck)
        B.evolve(7)
        b = B.download(dtype=dt)
        assert B.time == ta
    for q in range(4):
        assert np.array_equal(a[q], b[q]), q
