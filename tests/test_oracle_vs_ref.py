"""Oracle restatement against the reference's own sources compiled with the
project shims (only where oracle/_ref was built, i.e. next to a reference
checkout). Also runs the reference's own test programs on that build."""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib

REF = oracle_lib.load_ref(64)
pytestmark = pytest.mark.skipif(REF is None, reason="oracle/_ref not built (no reference checkout here)")


@pytest.mark.parametrize("nd,N,stencil", [(2, 64, 0), (2, 64, 3), (3, 24, 0), (3, 24, 2)])
def test_step(oracle, nd, N, stencil):
    rng = np.random.default_rng(nd * 100 + stencil)
    p = oracle_lib.make_params(NDIMS=nd, N=N, T0=4.0, stencil=stencil)
    f = [rng.standard_normal((N,) * nd) for _ in range(4)]
    a = oracle.evolve(p, *f, 10)
    b = REF.evolve(p, *f, 10)
    for q in range(4):
        assert np.abs(a[q] - b[q]).max() / np.abs(b[q]).max() <= 1e-13
    assert a[4] == b[4]


@pytest.mark.parametrize("nd,N,stencil", [(2, 64, 0), (2, 48, 2), (3, 24, 0), (3, 24, 1)])
def test_hamiltonian_step(oracle, nd, N, stencil):
    """vvsl_hamiltonian_form (s_integrate.cpp:358-395) against the oracle."""
    rng = np.random.default_rng(nd * 1000 + stencil + 7)
    p = oracle_lib.make_params(NDIMS=nd, N=N, T0=4.0, stencil=stencil)
    f = [rng.standard_normal((N,) * nd) for _ in range(4)]
    a = oracle.evolve(p, *f, 10, form=1)
    b = REF.evolve(p, *f, 10, form=1)
    for q in range(4):
        assert np.abs(a[q] - b[q]).max() / np.abs(b[q]).max() <= 1e-13
    assert a[4] == b[4]


@pytest.mark.parametrize("nd,N", [(2, 64), (2, 30), (3, 16), (3, 20)])
def test_spectral_laplacian(oracle, nd, N):
    """compute_laplacian_fft (s_integrate.cpp:179-296) against the oracle."""
    rng = np.random.default_rng(nd * 10 + N)
    p = oracle_lib.make_params(NDIMS=nd, N=N, dx=0.7, laplacian=1)
    f = rng.standard_normal((N,) * nd)
    a = oracle.laplacian(p, f)
    b = REF.laplacian_fft(p, f)
    assert np.abs(a - b).max() / np.abs(b).max() <= 1e-13


@pytest.mark.parametrize("nd,N,thr", [(2, 96, 1), (3, 20, 1), (3, 20, 50)])
def test_cores(oracle, nd, N, thr):
    rng = np.random.default_rng(N + thr)
    p = oracle_lib.make_params(NDIMS=nd, N=N, thr=thr)
    th = rng.uniform(-np.pi, np.pi, (N,) * nd)
    n1, mask = oracle.cores(p, th)
    n2, pos = REF.cores(p, th)
    offs = pos[:, 0] + N * pos[:, 1] if nd == 2 else (pos[:, 0] * N + pos[:, 1]) * N + pos[:, 2]
    assert n1 == n2
    assert np.array_equal(np.sort(offs), np.flatnonzero(mask.reshape(-1)))


@pytest.mark.parametrize("nd,N", [(2, 64), (3, 24)])
def test_powerspec(oracle, nd, N):
    rng = np.random.default_rng(3)
    p = oracle_lib.make_params(NDIMS=nd, N=N)
    fld = rng.standard_normal((N,) * nd)
    a = oracle.powerspec(p, fld)
    b = REF.powerspec(p, fld)
    assert np.array_equal(a[2], b[2])
    ok = b[2] > 0
    assert np.abs(a[0][ok] - b[0][ok]).max() / np.abs(b[0][ok]).max() <= 1e-12


@pytest.mark.parametrize("prog", ["ref_laplacian", "ref_fdm_matrix"])
def test_reference_test_programs_pass_on_shims(prog):
    path = os.path.join(oracle_lib.REF_DIR, prog)
    if not os.path.exists(path):
        pytest.skip("not built")
    assert subprocess.run([path]).returncode == 0
