"""The oracle pinned against the reference's own tests and fixtures
(CPU only): FFT against numpy, Philox known-answer vectors, the Laplacian
known-answer tests of src/tests/laplacian.cpp and src/tests/fdm_matrix.cpp,
and the golden states/masks/spectra generated from the reference's sources."""
import ctypes
import os

import numpy as np
import pytest

import oracle_lib
from strings_util import num_cores2_ascending

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("dims", [(8,), (12,), (96,), (160,), (30, 30), (16, 16, 16), (12, 20, 6), (96, 96)])
def test_fft_matches_numpy(oracle, dims):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
    assert np.abs(oracle.fftn(x, -1) - np.fft.fftn(x)).max() <= 1e-13 * np.abs(x).sum() ** 0.5 * 10
    b = oracle.fftn(x, +1)
    ref = np.fft.ifftn(x) * x.size
    assert np.abs(b - ref).max() / np.abs(ref).max() <= 1e-13


def test_philox_known_answers(oracle):
    f = oracle.lib.orc_philox
    f.argtypes = [ctypes.c_void_p] * 3
    f.restype = None
    kats = [  # Random123 philox4x32-10 known-answer vectors (ctr, key) -> out
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kats:
        c = np.array(ctr, dtype=np.uint32)
        k = np.array(key, dtype=np.uint32)
        o = np.zeros(4, dtype=np.uint32)
        f(c.ctypes.data, k.ctypes.data, o.ctypes.data)
        assert tuple(int(v) for v in o) == want


def test_normals_are_standard(oracle):
    z = np.array([oracle.normal(7, a, m) for a in range(4) for m in range(20000)])
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    assert oracle.normal(7, 0, 5) != oracle.normal(8, 0, 5)


def _wave(nd, N):
    L = N / 2.0
    i = np.arange(N)
    if nd == 2:
        jj, ii = np.meshgrid(i, i, indexing="ij")
        return np.sin(np.float32(np.pi / L) * ii) + np.cos(np.pi / L * jj), L
    I, J, K = np.meshgrid(i, i, i, indexing="ij")
    return np.sin(np.pi / L * I) + np.cos(np.pi / L * J) + np.sin(np.pi / L * K), L


@pytest.mark.parametrize("nd,N", [(2, 128), (2, 256), (3, 128), (3, 256)])
def test_laplacian_known_answers(oracle, nd, N):
    """src/tests/laplacian.cpp:13-87 / fdm_matrix.cpp:109-244: zeros -> 0,
    sin/cos waves (dx = 1, L = N/2) -> -(pi/L)^2 f within 1e-5."""
    p = oracle_lib.make_params(NDIMS=nd, N=N, dx=1.0)
    z = oracle.laplacian(p, np.zeros((N,) * nd))
    assert np.abs(z).max() <= 1e-30
    f, L = _wave(nd, N)
    lap = oracle.laplacian(p, f)
    assert np.abs(lap - (-(np.pi / L) ** 2) * f).max() <= 1e-5


def test_fdm_matrix_golden(oracle):
    """The exact 16x16 operator of the disabled test
    test_build_coefficient_matrix (src/tests/fdm_matrix.cpp:40-107)."""
    want = np.loadtxt(os.path.join(GOLD, "fdm_matrix_n4.txt"))
    p = oracle_lib.make_params(NDIMS=2, N=4, dx=1.0)
    A = np.zeros((16, 16))
    for c in range(16):
        e = np.zeros(16)
        e[c] = 1.0
        A[:, c] = oracle.laplacian(p, e.reshape(4, 4)).reshape(-1)
    assert np.array_equal(A, want)


@pytest.mark.parametrize("name", ["step_2d32", "step_3d16"])
def test_step_golden(oracle, name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    p = oracle_lib.make_params(NDIMS=int(z["nd"]), N=int(z["N"]), lam=float(z["lam"]), T0=float(z["T0"]),
                               dx=float(z["dx"]), dt=float(z["dt"]))
    s0 = oracle.init_thermal(p, int(z["seed"]))
    nd = int(z["nd"])
    for q in range(4):
        if nd == 3 and q >= 2:
            # the reference leaves the 3D k=0 phidot amplitude uninitialised
            # (init.cpp:377-378): a constant offset; the oracle uses 0
            d = s0[q] - z["s0"][q]
            assert np.abs(d - d.mean()).max() <= 1e-14
        else:
            assert np.abs(s0[q] - z["s0"][q]).max() <= 1e-15 * max(1.0, np.abs(z["s0"][q]).max())
    for key, n in [("s1", 1), ("s10", 10)]:
        o = oracle.evolve(p, *z["s0"], n)
        for q in range(4):
            ref = z[key][q]
            assert np.abs(o[q] - ref).max() / np.abs(ref).max() <= 1e-13, (key, q)
        assert o[4] == float(z["tau1" if n == 1 else "tau10"])
    pk = np.load(os.path.join(GOLD, "pk_" + name.split("_")[1] + ".npz"))
    o = oracle.evolve(p, *z["s0"], 10)
    mine = oracle.powerspec(p, o[1])
    assert np.array_equal(mine[2], pk["count"])
    ok = pk["count"] > 0
    assert np.abs(mine[0][ok] - pk["pk"][ok]).max() / np.abs(pk["pk"][ok]).max() <= 1e-12
    assert np.abs(mine[1][ok] - pk["ks"][ok]).max() / np.abs(pk["ks"][ok]).max() <= 1e-12


def test_strings_golden(oracle):
    files = sorted(f for f in os.listdir(GOLD) if f.startswith("strings_"))
    assert len(files) == 6
    for f in files:
        z = np.load(os.path.join(GOLD, f))
        nd, N, thr = int(z["nd"]), int(z["N"]), int(z["thr"])
        p = oracle_lib.make_params(NDIMS=nd, N=N, thr=thr)
        n, mask = oracle.cores(p, z["theta"])
        want = np.unpackbits(z["mask_bits"])[: mask.size].reshape(mask.shape)
        assert n == int(z["n"]), f
        assert np.array_equal(mask, want), f
        if nd == 2:
            assert oracle.num_cores2(N, mask) == int(z["num_cores_serial"])
            assert num_cores2_ascending(N, np.flatnonzero(mask)) == int(z["num_cores_serial"])


def _stencil_weight_sum(setting, nd):
    """Sum of the float stencil weights of build_coefficient_matrix
    (s_integrate.cpp:9-14): centre + 2 nd sum of the off-centre weights."""
    f = np.float32
    c = {0: [f(-2.0) * f(nd), f(1.0)],
         1: [f(-5.0) / f(2.0) * f(nd), f(4.0) / f(3.0), f(-1.0) / f(12.0)],
         2: [f(-49.0) / f(18.0) * f(nd), f(3.0) / f(2.0), f(-3.0) / f(20.0), f(1.0) / f(90.0)],
         3: [f(-205.0) / f(72.0) * f(nd), f(8.0) / f(5.0), f(-1.0) / f(5.0), f(8.0) / f(315.0), f(-1.0) / f(560.0)]}[setting]
    return float(c[0]) + 2 * nd * sum(float(x) for x in c[1:])


@pytest.mark.parametrize("nd,N", [(2, 24), (3, 12)])
@pytest.mark.parametrize("setting", [0, 1, 2, 3, "spectral"])
def test_laplacian_sums_to_weight_sum_times_field_sum(oracle, nd, N, setting):
    """On a periodic lattice every site is the neighbour of as many sites as
    the stencil has points, so sum_m L(m) = W/dx^2 sum_m f(m), W the sum of the
    stencil's weights (0 for 5 and 7 points, ~1e-7 for the float weights of
    radius 2-4; 0 for the spectral operator). The background means of the
    device rely on it: the Laplacian's share of mean(pi_n) is formed from
    mean(psi) instead of per site."""
    dx = 0.5
    spectral = setting == "spectral"
    p = oracle_lib.make_params(NDIMS=nd, N=N, dx=dx, stencil=0 if spectral else setting,
                               laplacian=1 if spectral else 0)
    f = np.random.default_rng(3).standard_normal((N,) * nd) + 0.7
    lap = oracle.laplacian(p, f)
    W = 0.0 if spectral else _stencil_weight_sum(setting, nd)
    assert abs(lap.sum() - W / dx ** 2 * f.sum()) <= 1e-12 * np.abs(lap).sum()
    if not spectral and setting > 0:
        assert W != 0.0   # the float weights leave a small remainder, so the term matters


@pytest.mark.parametrize("nd,N", [(2, 32), (3, 16)])
def test_spectral_laplacian_plane_wave(oracle, nd, N):
    """The spectral Laplacian of a lattice plane wave is exactly -k^2 times it,
    k = 2 pi n / (N dx), for every n below the Nyquist index."""
    dx = 0.5
    p = oracle_lib.make_params(NDIMS=nd, N=N, dx=dx, laplacian=1)
    idx = np.indices((N,) * nd)
    n = [3, 1, 2][:nd]
    phase = sum(2 * np.pi * ni * ix / N for ni, ix in zip(n, idx))
    f = np.cos(phase + 0.3)
    k2 = sum((2 * np.pi * ni / (N * dx)) ** 2 for ni in n)
    out = oracle.laplacian(p, f)
    assert np.abs(out + k2 * f).max() <= 1e-11 * k2


def test_fast_atan2_error_bound():
    """The string finder's float angle (fast_atan2 in csrc/axs_analysis.cu,
    re-evaluated here in float32 step by step) stays within 5e-7 rad of atan2
    in all four quadrants, with the ratio a = min/max anywhere within the fast
    division's 2 ulp: the float stage's 1e-5 decision margin relies on it."""
    import re
    src = open(os.path.join(oracle_lib.ROOT, "axion-strings_gb300", "csrc", "axs_analysis.cu")).read()
    body = re.search(r"kAtanC\[8\] = \{([^}]*)\}", src).group(1)
    c = np.array([float(t.strip().rstrip("f")) for t in body.split(",")], dtype=np.float32)
    assert c.size == 8
    rng = np.random.default_rng(5)
    ang = rng.uniform(-np.pi, np.pi, 400000)
    rad = rng.uniform(1e-3, 10.0, ang.size)
    y = (rad * np.sin(ang)).astype(np.float32)
    x = (rad * np.cos(ang)).astype(np.float32)
    ax, ay = np.abs(x), np.abs(y)
    mx, mn = np.maximum(ax, ay), np.minimum(ax, ay)
    a0 = (mn / mx).astype(np.float32)
    up = np.float32(np.inf)
    for shift in (-2, -1, 0, 1, 2):   # __fdividef: within 2 ulp of the rounded quotient
        a = a0.copy()
        for _ in range(abs(shift)):
            a = np.nextafter(a, up if shift > 0 else -up).astype(np.float32)
        s = (a * a).astype(np.float32)
        p = np.full_like(a, c[7])
        for k in range(6, -1, -1):
            p = (p.astype(np.float64) * s + c[k]).astype(np.float32)   # fmaf: one rounding
        r = (p * a).astype(np.float32)
        r = np.where(ay > ax, (np.float32(1.5707963267948966) - r).astype(np.float32), r)
        r = np.where(x < 0, (np.float32(3.1415926535897932) - r).astype(np.float32), r)
        r = np.copysign(r, y)
        err = np.abs(r.astype(np.float64) - np.arctan2(y.astype(np.float64), x.astype(np.float64)))
        assert err.max() <= 5e-7, (shift, err.max())


def _table(name, n):
    import re
    src = open(os.path.join(oracle_lib.ROOT, "axion-strings_gb300", "csrc", "axs_analysis.cu")).read()
    body = re.search(name + r"\[%d\] = \{([^}]*)\}" % n, src).group(1)
    c = np.array([float(t.strip().rstrip("f")) for t in body.split(",")], dtype=np.float32)
    assert c.size == n
    return c


def test_fast_turns_error_bound():
    """The string finder's float angle in turns (fast_turns, re-evaluated here
    in float32 step by step) stays within 3.3e-7 turns of atan2/(2 pi) in all
    four quadrants and on the axes, with the division anywhere within its 2
    ulp: the finder's 1e-5 decision margin rests on it (edge values within
    7e-7, a plaquette's sum of three within 2.3e-6)."""
    c = _table("kTurnC", 6)
    rng = np.random.default_rng(6)
    ang = np.concatenate([rng.uniform(-np.pi, np.pi, 400000), np.arange(-4, 5) * np.pi / 4])
    rad = np.concatenate([rng.uniform(1e-3, 10.0, 400000), np.full(9, 2.5)])
    y = (rad * np.sin(ang)).astype(np.float32)
    x = (rad * np.cos(ang)).astype(np.float32)
    y[-9:][[0, 4, 8]] = 0.0   # exact axes: y = 0 at x < 0 (both signs of zero) and x > 0
    y[-9] = -0.0
    x[-9:][[2, 6]] = 0.0
    ax, ay = np.abs(x), np.abs(y)
    mx, mn = np.maximum(ax, ay), np.minimum(ax, ay)
    a0 = (mn / mx).astype(np.float32)
    up = np.float32(np.inf)
    for shift in (-2, -1, 0, 1, 2):   # __fdividef: within 2 ulp of the rounded quotient
        a = a0.copy()
        for _ in range(abs(shift)):
            a = np.where(a > 0, np.nextafter(a, up if shift > 0 else -up), a).astype(np.float32)
        s = (a * a).astype(np.float32)
        p = np.full_like(a, c[5])
        for k in range(4, -1, -1):
            p = (p.astype(np.float64) * s + c[k]).astype(np.float32)   # fmaf: one rounding
        r = (p * a).astype(np.float32)
        r = np.where(ay > ax, (np.float32(0.25) - r).astype(np.float32), r)
        r = np.where(x < 0, (np.float32(0.5) - r).astype(np.float32), r)
        r = np.copysign(r, y)
        want = np.arctan2(y.astype(np.float64), x.astype(np.float64)) / (2 * np.pi)
        err = np.abs(r.astype(np.float64) - want)
        assert err.max() <= 3.3e-7, (shift, err.max())


def test_atan_tables_match_their_generator():
    """Both float atan tables are the output of tests/atan_fit.py (to the last
    float32 ulp, for BLAS rounding differences between machines)."""
    import atan_fit
    for name, gen in atan_fit.tables().items():
        c = _table(name, len(gen))
        g = gen.astype(np.float32)
        ulp = np.spacing(np.abs(g))
        assert np.all(np.abs(c - g) <= ulp), (name, c, g)


def test_fp64_angle_and_modulus_by_table_rotation():
    """The FP64 background means' |atan2(a, b)| and |(a, b)| (abs_phi_theta in
    axs_analysis.cu), restated in numpy: a float angle within 5e-7 rad picks
    the nearest k pi/128; the vector is rotated by it with double cosine and
    sine; the remainder angle and the modulus come from series in u = y/x,
    which stays below 0.0125 (tan(pi/256 + 5e-7) = 0.01227). Within 4 ulp of
    arctan2 and sqrt, the truncated series' terms below 3e-17."""
    assert np.tan(np.pi / 256 + 5e-7) < 0.0125
    u = 0.0125
    assert u ** 9 / 9 < 1e-18 and 5 * (u * u) ** 4 / 128 < 3e-17
    rng = np.random.default_rng(3)
    n = 400000
    a = rng.standard_normal(n) * np.exp(rng.uniform(-12, 12, n))
    b = rng.standard_normal(n) * np.exp(rng.uniform(-12, 12, n))
    a[:200], b[200:400], b[400:600], a[400:600] = 0.0, 0.0, -1.0, rng.standard_normal(200) * 1e-13
    t0 = np.arctan2(a.astype(np.float32), b.astype(np.float32))
    t0 = t0 + rng.uniform(-5e-7, 5e-7, n).astype(np.float32)   # the float angle's error
    k = np.rint(t0 * np.float32(128 / np.pi)).astype(np.int64)
    th = k * (np.pi / 128.0)
    c, s = np.cos(th), np.sin(th)
    x, y = b * c + a * s, a * c - b * s
    uu = y / x
    assert np.all(x > 0) and np.abs(uu).max() < 0.0125
    u2 = uu * uu
    t = (uu * u2) * ((u2 * (-1 / 7) + 1 / 5) * u2 - 1 / 3) + uu + th
    t = np.where(t > np.pi, t - 2 * np.pi, np.where(t < -np.pi, t + 2 * np.pi, t))
    mod = x * (u2 * ((u2 * (1 / 16) - 1 / 8) * u2 + 0.5) + 1.0)
    ref_t, ref_m = np.abs(np.arctan2(a, b)), np.sqrt(a * a + b * b)
    assert np.abs(np.abs(t) - ref_t).max() <= 4 * np.spacing(np.pi)
    assert (np.abs(mod - ref_m) / ref_m).max() <= 4 * np.spacing(1.0)
