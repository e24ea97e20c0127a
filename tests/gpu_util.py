"""Shared helpers of the GPU parity tests."""
import numpy as np

import oracle_lib


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)


def params(axs, nd=3, N=32, precision=64, **kw):
    base = dict(NDIMS=nd, N=N, T_initial=4.0, space_step=0.5, time_step=0.1, stencil_setting=0,
                precision=precision, thr=1, prs=1)
    base.update(kw)
    return axs.default_params(**base)


def orc(p):
    return oracle_lib.from_axs(p)
