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
