"""Error behaviour of the C ABI (host-side fault injection only)."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


def test_invalid_parameters_are_rejected(axs):
    for bad in [dict(N=31), dict(NDIMS=4), dict(stencil_setting=7), dict(precision=16), dict(N=2), dict(N=4098),
                dict(nd=2, N=32770)]:
        with pytest.raises(axs.AxsError) as e:
            axs.Lattice(params(axs, **{"nd": 3, "N": 32, "precision": 64, **bad}))
        assert e.value.code == axs.ERR_ARG


def test_out_of_device_memory_is_an_error_not_a_crash(axs):
    with pytest.raises(axs.AxsError) as e:
        axs.Lattice(params(axs, 3, 4096, 64))
    assert e.value.code in (axs.ERR_NOMEM, axs.ERR_ARG)


def test_positions_before_find_is_a_state_error(axs):
    with axs.Lattice(params(axs, 3, 16, 64)) as L:
        with pytest.raises(axs.AxsError) as e:
            L.string_positions()
        assert e.value.code == axs.ERR_STATE


def test_wrong_array_size(axs):
    with axs.Lattice(params(axs, 3, 16, 64)) as L:
        with pytest.raises(ValueError):
            L.upload(np.zeros(10))
