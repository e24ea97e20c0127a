"""Parity at the sizes of the configured workloads, on the kernels the
autotuner picks for them (nothing forced unless a test says so):

  2D 512^2 FP64, 5-point Laplacian, plaquette count (the CPU-runnable case);
  3D 256^3 FP64, 7-point Laplacian, strings and the 128-bin axion spectrum;
  3D 256^3 FP32 on the two-step z-march kernels against the FP64 run.

References: vvsl_field_rescaled (src/standard/s_integrate.cpp:305-348),
cores2/cores3 (src/common/string_finding.cpp:3-86), output_powerspec
(src/common/pk_estimation.cpp:37-214). Tolerances: FP64 fields within 1e-12
of the oracle after 10 steps (max-norm relative); output_powerspec bins
within 1e-11, axion spectrum bins within 1e-10; string masks from psi equal
to the oracle's on numpy's atan2 of the same field except at cells whose
plaquette sum lies within 1e-12 of the threshold (an ulp of atan2 can move
those); FP32 fields within 1e-5 of FP64 after 10 steps."""
import os

import numpy as np
import pytest

from gpu_util import orc, params, rel
from strings_util import accept_value, threshold_only_mismatches

pytestmark = pytest.mark.gpu

# (name, T_initial, prs, start): the reference's own thermal start with its
# PRS step, and the configured flat k_cut = 1 start with the unrescaled
# coupling (phi'' + (2/tau) phi' - lap phi + tau^2 lambda phi (|phi|^2 - 1) = 0)
STARTS = [("thermal", 4.0, 1), ("flat", 0.0, 0)]


def _start(oracle, op, kind, seed):
    return oracle.init_thermal(op, seed) if kind == "thermal" else oracle.init_flat(op, seed, 1.0)


def _strings_check(axs, oracle, p, op, g, L, nd):
    """Mask from psi on the device vs the oracle on host atan2."""
    n_g, c_g, mask_g = L.find_strings(want_mask=True)
    theta = np.arctan2(np.asarray(g[0], np.float64), np.asarray(g[1], np.float64))
    n_o, mask_o = oracle.cores(op, theta)
    nmis, ok = threshold_only_mismatches(nd, theta, mask_g, mask_o, accept_value(p.thr))
    print("strings from psi: flagged", n_o, "mismatches", nmis)
    assert ok, "a mask difference away from the threshold"
    assert n_g == int(np.count_nonzero(mask_g))
    if nd == 2 and nmis == 0:
        assert c_g == oracle.num_cores2(p.N, mask_o)
    return n_g


@pytest.mark.parametrize("kind,T0,prs", STARTS)
def test_2d_512_fp64(axs, oracle, kind, T0, prs):
    p = params(axs, 2, 512, 64, T_initial=T0, prs=prs)
    op = orc(p)
    f = _start(oracle, op, kind, 5)
    with axs.Lattice(p) as L:
        if kind == "flat":
            L.init_flat(5, 1.0)
            gi = L.download()
            for q in range(4):
                assert rel(gi[q], f[q]) <= 1e-12, ("init", q, rel(gi[q], f[q]))
        L.upload(*f)
        L.evolve(10)
        g = L.download()
        tau, steps = L.time
        print("2D 512^2", kind, L.describe())
        o = oracle.evolve(op, *f, 10)
        for q in range(4):
            assert rel(g[q], o[q]) <= 1e-12, (q, rel(g[q], o[q]))
        assert steps == 10 and tau == o[4]
        _strings_check(axs, oracle, p, op, g, L, 2)
        pk, ks, cnt = L.powerspec(axs.PHI2)
    pko, kso, cnto = oracle.powerspec(op, g[1])
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-11 and rel(ks[ok], kso[ok]) <= 1e-11


def test_2d_512_fp64_plaquette_cadence(axs, oracle):
    """The count every 100 steps over 300 steps of the reference's PRS step
    from the thermal start: each count equals the oracle's on host atan2 of
    the device field up to threshold cells (the fields themselves are
    compared at the end)."""
    p = params(axs, 2, 512, 64)
    op = orc(p)
    f = oracle.init_thermal(op, 9)
    o = list(f)
    with axs.Lattice(p) as L:
        L.upload(*f)
        for block in range(3):
            L.evolve(100)
            g = L.download()
            _strings_check(axs, oracle, p, op, g, L, 2)
        ot = oracle.evolve(op, *o, 300)
    for q in range(4):
        # 300 steps: rounding differences grow (a 1e-16 perturbation of the
        # start grows to ~1e-13 in the oracle itself)
        assert rel(g[q], ot[q]) <= 1e-11, (q, rel(g[q], ot[q]))


@pytest.mark.parametrize("kind,T0,prs", STARTS)
def test_3d_256_fp64(axs, oracle, kind, T0, prs):
    p = params(axs, 3, 256, 64, T_initial=T0, prs=prs)
    op = orc(p)
    f = _start(oracle, op, kind, 3)
    with axs.Lattice(p) as L:
        if kind == "flat":
            L.init_flat(3, 1.0)
            gi = L.download()
            for q in range(4):
                assert rel(gi[q], f[q]) <= 1e-12, ("init", q, rel(gi[q], f[q]))
        L.upload(*f)
        L.evolve(10)
        g = L.download()
        tau, steps = L.time
        print("3D 256^3", kind, L.describe())
        o = oracle.evolve(op, *f, 10)
        for q in range(4):
            assert rel(g[q], o[q]) <= 1e-12, (q, rel(g[q], o[q]))
        assert steps == 10 and tau == o[4]
        _strings_check(axs, oracle, p, op, g, L, 3)
        k, apk, acnt = L.axion_spectrum(128)
        pk, ks, cnt = L.powerspec(axs.PHI2)
    ko, apko, acnto = oracle.axion_spectrum(op, *g, tau, 128)
    assert np.array_equal(acnt, acnto)
    ok = acnto > 0
    assert rel(apk[ok], apko[ok]) <= 1e-10 and rel(k[ok], ko[ok]) <= 1e-12
    pko, kso, cnto = oracle.powerspec(op, g[1])
    assert np.array_equal(cnt, cnto)
    ok = cnto > 0
    assert rel(pk[ok], pko[ok]) <= 1e-11


@pytest.mark.parametrize("force", [None, "1,30,128", "1,39,256"])
def test_3d_256_fp32_two_step_against_fp64(axs, oracle, force):
    """FP32 on the autotuned kernel and on the two-step kernels of the
    1024^3 headline (variant 30) and of the ensemble (variant 39), against
    the FP64 GPU run (itself within 1e-12 of the oracle above), after 10
    steps from the configured flat start with the unrescaled coupling."""
    p64 = params(axs, 3, 256, 64, T_initial=0.0, prs=0)
    p32 = params(axs, 3, 256, 32, T_initial=0.0, prs=0)
    f = oracle.init_flat(orc(p64), 4, 1.0)
    prev = os.environ.get("AXS_FORCE_CONFIG")
    if force:
        os.environ["AXS_FORCE_CONFIG"] = force
    try:
        with axs.Lattice(p32) as B:
            B.upload(*f)
            B.evolve(10)
            d = B.describe()
            gb = B.download()
            n32, _, _ = B.find_strings()
    finally:
        if prev is None:
            os.environ.pop("AXS_FORCE_CONFIG", None)
        else:
            os.environ["AXS_FORCE_CONFIG"] = prev
    print("3D 256^3 FP32", d)
    if force:
        assert "two steps per pass" in d, d
    with axs.Lattice(p64) as A:
        A.upload(*f)
        A.evolve(10)
        ga = A.download()
        n64, _, _ = A.find_strings()
    for q in range(4):
        assert rel(gb[q], ga[q]) <= 1e-5, (q, rel(gb[q], ga[q]))
    # string counts of the FP32 and FP64 fields: same network to 1e-3
    assert abs(n32 - n64) <= max(10, n64 // 1000), (n32, n64)
