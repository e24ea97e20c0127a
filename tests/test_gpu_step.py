"""Parity of the fused leapfrog step against the oracle restatement of
vvsl_field_rescaled (src/standard/s_integrate.cpp:305-348).

Tolerance: FP64 fields within 1e-12 relative (max-norm) after 10 steps; the
reference's own operation order differs only by rounding."""
import os

import numpy as np
import pytest

from gpu_util import orc, params, rel

pytestmark = pytest.mark.gpu

CASES = [
    (2, 64, 0, 1), (2, 48, 2, 1), (2, 64, 3, 0),
    (3, 32, 0, 1), (3, 24, 1, 1), (3, 64, 0, 1), (3, 40, 0, 1), (3, 48, 0, 0), (3, 32, 3, 1),
]


@pytest.mark.parametrize("nd,N,stencil,prs", CASES)
def test_fp64_matches_oracle_after_10_steps(axs, oracle, nd, N, stencil, prs):
    p = params(axs, nd, N, 64, stencil_setting=stencil, prs=prs)
    op = orc(p)
    f = oracle.init_thermal(op, 11)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(10)
        g = L.download()
        tau, steps = L.time
    o = oracle.evolve(op, *f, 10)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-12, (q, rel(g[q], o[q]))
    assert steps == 10
    assert tau == o[4]


def test_single_steps_and_graph_replays_agree(axs, oracle):
    p = params(axs, 3, 32, 64)
    op = orc(p)
    f = oracle.init_thermal(op, 3)
    with axs.Lattice(p) as A, axs.Lattice(p) as B:
        A.upload(*f)
        B.upload(*f)
        for _ in range(12):
            A.evolve(1)
        B.evolve(4)
        B.evolve(4)
        B.evolve(4)
        ga, gb = A.download(), B.download()
    for q in range(4):
        assert np.array_equal(ga[q], gb[q])


@pytest.mark.parametrize("precision", [32, 64])
def test_kernel_variants_bit_identical(axs, oracle, precision):
    """The generic per-site kernel and every TMA z-march configuration share
    one per-site update, so autotuning never changes results."""
    p = params(axs, 3, 64, precision)
    op = orc(p)
    f = oracle.init_thermal(op, 5)
    outs = []
    for force in ["0,0,64", "1,0,32", "1,1,64", "1,2,64", "1,3,128", "1,4,32",
                  "1,5,64", "1,6,32", "1,7,64", "1,8,128", "1,9,16", "1,16,32", "1,27,64", "1,38,32"]:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.upload(*f)
                L.evolve(7)
                outs.append((L.describe(), L.download()))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    d0, g0 = outs[0]
    for d, g in outs[1:]:
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), (d0, d, q)


TWO_STEP = ["1,10,32", "1,11,64", "1,12,128", "1,13,16", "1,14,64", "1,15,128", "1,17,32", "1,18,64",
            "1,19,128", "1,28,32", "1,29,64", "1,30,32", "1,31,64", "1,39,32", "1,40,64"]


@pytest.mark.parametrize("N", [64, 160])
def test_two_step_variants_bit_identical(axs, N):
    """Two steps per pass (halo depth 2) give the bits of two one-step passes:
    even and odd intervals (the odd step runs on the one-step partner), eager
    launches and graph replays, one x tile (N=64) and two (N=160, tx=80)."""
    p = params(axs, 3, N, 32)
    outs = []
    for force in ["0,0,64", "1,6,64"] + TWO_STEP:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.init_thermal(21)
                for n in (1, 3, 1, 6, 2, 5):
                    L.evolve(n)
                d = L.describe()
                outs.append((force, d, L.download(dtype=np.float32), L.time))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    f0, d0, g0, t0 = outs[0]
    assert "generic" in d0
    for force, d, g, t in outs[1:]:
        if force in TWO_STEP:
            assert "two steps per pass" in d, d
        assert t == t0, (d, t, t0)
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), (d0, d, q)


THREE_STEP = ["1,46,64", "1,46,32", "1,47,64", "1,47,128"]


@pytest.mark.parametrize("N", [160, 192])
def test_three_step_variants_bit_identical(axs, N):
    """Three steps per pass (halo depth 3) give the bits of one-step passes:
    intervals of every length mod 3 (the last one or two steps run on the
    two-step and one-step partners), eager launches and graph replays."""
    p = params(axs, 3, N, 32)
    outs = []
    for force in ["0,0,64"] + THREE_STEP:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.init_thermal(23)
                for n in (1, 3, 1, 6, 2, 5, 4, 3):
                    L.evolve(n)
                d = L.describe()
                outs.append((force, d, L.download(dtype=np.float32), L.time))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    f0, d0, g0, t0 = outs[0]
    assert "generic" in d0
    for force, d, g, t in outs[1:]:
        assert "three steps per pass" in d, d
        assert t == t0, (d, t, t0)
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), (d0, d, q)


def test_two_step_after_analysis_and_checkpoint(axs):
    """The momentum moves between two buffers in two-step mode; analysis
    (which uses the spare buffer), checkpoints and uploads in between keep
    the run identical to the one-step run."""
    p = params(axs, 3, 160, 32)
    res = []
    for force in ["1,6,64", "1,10,64", "1,30,64", "1,46,64", "1,47,32"]:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.init_thermal(8)
                L.evolve(5)
                a = L.download(dtype=np.float32)
                n1, _, _ = L.find_strings()
                e1 = L.energies()
                ck = L.checkpoint()
                L.evolve(4)
                L.restore(ck)
                L.evolve(3)
                pk = L.axion_spectrum(16)
                L.evolve(2)
                res.append((a, n1, e1, pk, L.download(dtype=np.float32), L.time))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    (a0, n0, e0, pk0, g0, t0) = res[0]
    for (a1, n1, e1, pk1, g1, t1) in res[1:]:
        assert n0 == n1 and t0 == t1
        assert np.array_equal(np.asarray(e0), np.asarray(e1))
        for x, y in zip(pk0, pk1):
            assert np.array_equal(x, y)
        for q in range(4):
            assert np.array_equal(a0[q], a1[q])
            assert np.array_equal(g0[q], g1[q])


def test_fp32_error_against_fp64(axs, oracle):
    """FP32 fields after 10 steps from the identical (rounded) start stay
    within 1e-5 relative of the FP64 run."""
    p64 = params(axs, 3, 64, 64)
    p32 = params(axs, 3, 64, 32)
    f = oracle.init_thermal(orc(p64), 9)
    with axs.Lattice(p64) as A, axs.Lattice(p32) as B:
        A.upload(*f)
        B.upload(*f)
        A.evolve(10)
        B.evolve(10)
        ga, gb = A.download(), B.download()
    for q in range(4):
        assert rel(gb[q], ga[q]) <= 1e-5, (q, rel(gb[q], ga[q]))


def test_initial_drift_is_reference_first_step(axs, oracle):
    """The first step after an upload is a pure drift, as the reference's
    zeroed ker_curr makes it (s_run.cpp:44-47, s_integrate.cpp:313)."""
    p = params(axs, 2, 32, 64)
    op = orc(p)
    f = oracle.init_thermal(op, 2)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(1)
        g = L.download()
    o = oracle.evolve(op, *f, 1)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-13


def test_literal_equation_stays_finite_short(axs, oracle):
    """prs = 0 (lambda without 1/tau^2) on a flat k_cut field: 10 steps."""
    p = params(axs, 3, 64, 64, prs=0, T_initial=0.0, lambda_=1.0)
    op = orc(p)
    f = oracle.init_flat(op, 4, 1.0)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(10)
        g = L.download()
        assert L.check_finite()
    o = oracle.evolve(op, *f, 10)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-12


@pytest.mark.parametrize("nd,N,stencil", [(2, 64, 0), (2, 48, 1), (3, 32, 0), (3, 24, 2), (3, 40, 0)])
def test_hamiltonian_form_matches_oracle(axs, oracle, nd, N, stencil):
    """form = 1: vvsl_hamiltonian_form (s_integrate.cpp:358-395), FP64 within
    1e-12 of the oracle (itself pinned to the reference's compiled function)."""
    p = params(axs, nd, N, 64, stencil_setting=stencil, form=1)
    op = orc(p)
    f = oracle.init_thermal(op, 13)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(10)
        g = L.download()
        tau, steps = L.time
    o = oracle.evolve(op, *f, 10, form=1)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-12, (q, rel(g[q], o[q]))
    assert tau == o[4] and steps == 10


@pytest.mark.parametrize("N", [64, 160])
def test_hamiltonian_form_kernels_bit_identical(axs, N):
    """The generic, one-step and two-step kernels give the same bits in form 1."""
    p = params(axs, 3, N, 32, form=1)
    outs = []
    for force in ["0,0,64", "1,6,64", "1,10,128", "1,17,32"]:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.init_thermal(4)
                for n in (1, 4, 3):
                    L.evolve(n)
                outs.append((L.describe(), L.download(dtype=np.float32)))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    d0, g0 = outs[0]
    for d, g in outs[1:]:
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), (d0, d, q)


def test_hamiltonian_form_rejects_rescaled_analyses(axs):
    p = params(axs, 3, 32, 64, form=1)
    with axs.Lattice(p) as L:
        L.init_thermal(1)
        with pytest.raises(axs.AxsError):
            L.energies()
        with pytest.raises(axs.AxsError):
            L.axion_spectrum(16)


@pytest.mark.parametrize("nd,N,form", [(2, 64, 0), (3, 32, 0), (3, 24, 1), (2, 48, 1)])
def test_spectral_step_matches_oracle(axs, oracle, nd, N, form):
    """laplacian = 1 (the reference's compute_laplacian_fft branch of
    vvsl_field_rescaled, s_integrate.cpp:327-329), FP64 after 10 steps within
    1e-11 of the oracle (the transforms differ from the oracle's by rounding)."""
    p = params(axs, nd, N, 64, laplacian=1, form=form)
    op = orc(p)
    f = oracle.init_thermal(op, 17)
    with axs.Lattice(p) as L:
        L.upload(*f)
        L.evolve(4)
        L.evolve(6)
        g = L.download()
        tau, steps = L.time
    o = oracle.evolve(op, *f, 10, form=form)
    for q in range(4):
        assert rel(g[q], o[q]) <= 1e-11, (q, rel(g[q], o[q]))
    assert tau == o[4] and steps == 10


def test_spectral_step_fp32_against_fp64(axs, oracle):
    p64 = params(axs, 3, 48, 64, laplacian=1)
    p32 = params(axs, 3, 48, 32, laplacian=1)
    f = oracle.init_thermal(orc(p64), 19)
    with axs.Lattice(p64) as A, axs.Lattice(p32) as B:
        A.upload(*f)
        B.upload(*f)
        A.evolve(10)
        B.evolve(10)
        ga, gb = A.download(), B.download()
    for q in range(4):
        assert rel(gb[q], ga[q]) <= 1e-5, (q, rel(gb[q], ga[q]))


def test_spectral_after_finite_difference_lattice_of_same_shape(axs, oracle):
    """A finite-difference lattice tunes (and caches) a z-march configuration
    for its shape; a spectral lattice of the same shape and precision created
    afterwards still takes the spectral step (the tuning is keyed by the
    Laplacian too): it agrees with an FP64 spectral run from the same start
    (the finite-difference step would differ at the 1e-2 level)."""
    N = 128
    with axs.Lattice(params(axs, 3, N, 32)) as F:
        F.init_thermal(3)
        F.evolve(4)
    f = oracle.init_thermal(orc(params(axs, 3, N, 64, laplacian=1)), 23)
    with axs.Lattice(params(axs, 3, N, 32, laplacian=1)) as B, \
            axs.Lattice(params(axs, 3, N, 64, laplacian=1)) as A:
        for L in (A, B):
            L.upload(*f)
            L.evolve(10)
            assert "spectral" in L.describe(), L.describe()
        ga, gb = A.download(), B.download()
    for q in range(4):
        assert rel(gb[q], ga[q]) <= 1e-5, (q, rel(gb[q], ga[q]))


RADIUS_VARIANTS = {1: ["1,20,32", "1,21,64", "1,32,64", "1,33,16", "1,41,64", "1,41,32", "1,45,64", "1,48,64",
                        "1,49,32", "1,50,64", "1,57,32"],
                   2: ["1,22,64", "1,23,128", "1,34,32", "1,35,16", "1,42,32", "1,43,64", "1,51,32", "1,52,64",
                       "1,53,16"],
                   3: ["1,24,32", "1,25,64", "1,26,16", "1,36,16", "1,37,64", "1,44,32", "1,54,32", "1,55,16",
                       "1,56,64"]}


@pytest.mark.parametrize("stencil", [1, 2, 3])
@pytest.mark.parametrize("N,precision", [(64, 32), (160, 32), (64, 64), (160, 64)])
def test_higher_order_zmarch_bit_identical(axs, stencil, N, precision):
    """The TMA z-march kernels for stencil radius 2..4 give the generic
    kernel's bits (same stencil association order), with and without x tiling."""
    p = params(axs, 3, N, precision, stencil_setting=stencil)
    dt = np.float32 if precision == 32 else np.float64
    outs = []
    for force in ["0,0,64"] + RADIUS_VARIANTS[stencil]:
        os.environ["AXS_FORCE_CONFIG"] = force
        try:
            with axs.Lattice(p) as L:
                L.init_thermal(31)
                for n in (1, 4, 3):
                    L.evolve(n)
                outs.append((L.describe(), L.download(dtype=dt)))
        finally:
            del os.environ["AXS_FORCE_CONFIG"]
    d0, g0 = outs[0]
    assert "generic" in d0
    if precision == 32:
        assert all("stencil radius %d" % (stencil + 1) in d for d, _ in outs[1:]), [d for d, _ in outs]
    for d, g in outs[1:]:
        for q in range(4):
            assert np.array_equal(g[q], g0[q]), (d0, d, q)
