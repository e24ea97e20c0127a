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
                  "1,5,64", "1,6,32", "1,7,64", "1,8,128", "1,9,16"]:
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
