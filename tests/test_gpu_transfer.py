"""Host <-> device transfers: pageable arrays go through chunked, double-
buffered staging; page-locked arrays are read and written by the packing
kernels directly. Round trips are exact (up to rounding to the lattice
precision)."""
import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("host", [np.float32, np.float64])
def test_round_trip_multi_chunk_pageable(axs, precision, host):
    N = 336   # 37.9 M sites: more than one 32 M-element staging chunk
    p = params(axs, 3, N, precision)
    rng = np.random.default_rng(precision)
    f = [rng.standard_normal((N, N, N)).astype(host) for _ in range(4)]
    with axs.Lattice(p) as L:
        L.upload(*f, dtype=host)
        g = L.download(dtype=host)
    lat = np.float32 if precision == 32 else np.float64
    for q in range(4):
        assert np.array_equal(g[q], f[q].astype(lat).astype(host))


@pytest.mark.parametrize("precision", [32, 64])
def test_round_trip_page_locked(axs, precision):
    N = 64
    p = params(axs, 3, N, precision)
    dt = np.float32 if precision == 32 else np.float64
    bufs = [axs.PinnedBuffer((N, N, N), dt) for _ in range(4)]
    outs = [axs.PinnedBuffer((N, N, N), dt) for _ in range(4)]
    rng = np.random.default_rng(7)
    for b in bufs:
        b.array[...] = rng.standard_normal((N, N, N))
    with axs.Lattice(p) as L:
        L.upload(*[b.array for b in bufs], dtype=dt)
        fn = axs._lib.axs_download_f32 if precision == 32 else axs._lib.axs_download
        axs._check(fn(L._h, *[o.array.ctypes.data for o in outs]))
    for b, o in zip(bufs, outs):
        assert np.array_equal(b.array, o.array)
        b.free()
        o.free()


@pytest.mark.parametrize("precision", [32, 64])
def test_round_trip_page_locked_unaligned(axs, precision):
    """Page-locked arrays that start off a 16-byte boundary take the packing
    kernels' one-site-per-thread form instead of the 16-byte one."""
    N = 32
    n = N ** 3
    p = params(axs, 3, N, precision)
    dt = np.float32 if precision == 32 else np.float64
    bufs = [axs.PinnedBuffer((n + 1,), dt) for _ in range(4)]
    outs = [axs.PinnedBuffer((n + 1,), dt) for _ in range(4)]
    ins = [b.array[1:] for b in bufs]
    got = [o.array[1:] for o in outs]
    rng = np.random.default_rng(9)
    for v in ins:
        v[...] = rng.standard_normal(n)
    with axs.Lattice(p) as L:
        L.upload(*ins, dtype=dt)
        fn = axs._lib.axs_download_f32 if precision == 32 else axs._lib.axs_download
        axs._check(fn(L._h, *[v.ctypes.data for v in got]))
    for v, o in zip(ins, got):
        assert np.array_equal(v, o)
    for b in bufs + outs:
        b.free()


def test_single_field_transfers(axs):
    N = 32
    p = params(axs, 3, N, 64)
    rng = np.random.default_rng(1)
    f = [rng.standard_normal((N, N, N)) for _ in range(4)]
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.upload(None, f[0], None, None)          # one component of the psi pair
        g = L.download(fields=(True, False, False, True))
    assert np.array_equal(g[0], f[0])
    assert g[1] is None and g[2] is None
    assert np.array_equal(g[3], f[3])


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("host", ["pageable", "page-locked"])
def test_upload_forms_the_first_drift(axs, precision, form, host):
    """A full upload (psi and pi) forms the fresh state's first step, a pure
    drift, while the momentum packs; the evolution from it equals, bit for
    bit, the one that drifts in its first step (a state uploaded in parts),
    and one whose time was reset after the upload."""
    N = 48
    p = params(axs, 3, N, precision, form=form)
    dt = np.float32 if precision == 32 else np.float64
    rng = np.random.default_rng(11 + form)
    f = [rng.standard_normal((N, N, N)).astype(dt) for _ in range(4)]
    pinned = []
    if host == "page-locked":
        pinned = [axs.PinnedBuffer((N, N, N), dt) for _ in range(4)]
        for b, a in zip(pinned, f):
            b.array[...] = a
        f = [b.array for b in pinned]
    outs = []
    for mode in ("whole", "parts", "set_time"):
        with axs.Lattice(p) as L:
            L.init_flat(3, 1.0)
            L.evolve(2)   # tuned before the upload, so the tuner's trials leave the drift alone
            tau, steps = L.time
            if mode == "parts":
                L.upload(f[0], f[1], None, None, dtype=dt)
                L.upload(None, None, f[2], f[3], dtype=dt)
            else:
                L.upload(*f, dtype=dt)
            if mode == "set_time":
                L.set_time(tau, steps)
            L.evolve(5)
            outs.append((L.time, L.download(dtype=dt)))
    for b in pinned:
        b.free()
    (t0, g0) = outs[0]
    for t, g in outs[1:]:
        assert t == t0
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), q
