"""Separate lattice handles driven from different host threads. A handle is
not thread-safe, but handles share process-wide state (the autotuner's
cache, the transfer staging map, cached device queries): two threads each
tuning, evolving, analysing and transferring their own lattice give the
results of the same runs made one after the other."""
import threading

import numpy as np
import pytest

from gpu_util import params

pytestmark = pytest.mark.gpu


def _run(axs, N, seed, out, errors):
    try:
        p = params(axs, 3, N, 32, T_initial=0.0)
        with axs.Lattice(p) as L:
            L.init_flat(seed, 1.0)
            L.evolve(6)
            n, _, _ = L.find_strings()
            k, pk, cnt = L.axion_spectrum(16)
            host = [np.zeros(L.shape, np.float32) for _ in range(4)]
            L.upload(*host, dtype=np.float32)   # pageable transfer path (staging map)
            g = L.download(dtype=np.float32)
            out[(N, seed)] = (n, pk, g)
    except Exception as e:   # reported by the main thread
        errors.append(e)


def test_two_threads_two_lattices(axs):
    specs = [(80, 3), (112, 4)]   # sizes no other test tunes: both threads autotune at once
    threaded, errors = {}, []
    ts = [threading.Thread(target=_run, args=(axs, N, s, threaded, errors)) for N, s in specs]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    serial = {}
    for N, s in specs:
        _run(axs, N, s, serial, errors)
    assert not errors, errors
    for key in serial:
        n0, pk0, g0 = serial[key]
        n1, pk1, g1 = threaded[key]
        assert n0 == n1
        assert np.array_equal(pk0, pk1)
        for q in range(4):
            assert np.array_equal(g0[q], g1[q]), (key, q)
