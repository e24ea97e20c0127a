"""theta fields for string-finder parity: uniform random, and random with
many plaquette sums pushed to within a few ulp of the acceptance threshold."""
import numpy as np


def accept_value(thr):
    """(double)(0.5f * (1.0f - thr/100.0f)) of string_finding.cpp:8,40."""
    return float(np.float32(0.5) * (np.float32(1.0) - np.float32(thr) / np.float32(100.0)))


def near_threshold_theta(rng, nd, N, accept, frac=0.3):
    th = rng.uniform(-np.pi, np.pi, (N,) * nd)
    flat_n = ((th + np.pi) / (2 * np.pi)).reshape(-1)
    cells = rng.choice(flat_n.size, int(frac * flat_n.size / 4), replace=False)

    def c(a, b):
        return min(abs(b - a), 1 - abs(b - a))

    for m in cells:
        if nd == 2:
            i, j = m % N, m // N
            o = [i + N * j, (i + 1) % N + N * j, (i + 1) % N + N * ((j + 1) % N), i + N * ((j + 1) % N)]
        else:
            x, y, z = m % N, (m // N) % N, m // (N * N)
            o = [m, ((z + 1) % N) * N * N + y * N + x, ((z + 1) % N) * N * N + ((y + 1) % N) * N + x,
                 z * N * N + ((y + 1) % N) * N + x]
        t3 = accept - c(flat_n[o[0]], flat_n[o[1]]) - c(flat_n[o[1]], flat_n[o[2]])
        if 0 < t3 < 0.5:
            flat_n[o[3]] = (flat_n[o[2]] + t3) % 1.0
    return flat_n.reshape(th.shape) * 2 * np.pi - np.pi


def cell_sums3(n, z, y, x):
    """The three loop sums of cores3 (string_finding.cpp:34-86) for the cell
    with corner (i, j, k) = (z, y, x) of the normalised angles n."""
    N = n.shape[0]
    zp, yp, xp = (z + 1) % N, (y + 1) % N, (x + 1) % N

    def c(a, b):
        return min(abs(b - a), 1 - abs(b - a))

    d000, d100, d110 = n[z, y, x], n[zp, y, x], n[zp, yp, x]
    d010, d011, d001 = n[z, yp, x], n[z, yp, xp], n[z, y, xp]
    return np.array([c(d000, d100) + c(d100, d110) + c(d110, d010),
                     c(d000, d100) + c(d100, d011) + c(d011, d001),
                     c(d000, d010) + c(d010, d011) + c(d011, d001)])


def cell_sum2(n, j, i):
    """The loop sum of cores2 (string_finding.cpp:3-33) for the cell with
    corner (i, j) of the normalised angles n (array index [j, i])."""
    N = n.shape[0]
    ip, jp = (i + 1) % N, (j + 1) % N

    def c(a, b):
        return min(abs(b - a), 1 - abs(b - a))

    n1, n2, n3, n4 = n[j, i], n[j, ip], n[jp, ip], n[jp, i]
    return c(n1, n2) + c(n2, n3) + c(n3, n4)


def threshold_only_mismatches(nd, theta, mask_a, mask_b, accept, margin=1e-12):
    """Cells where two masks differ, and whether every one of them has a
    plaquette sum within `margin` of the acceptance value (a cell that an
    ulp of atan2 can move across the threshold)."""
    n = (theta + np.pi) / (2 * np.pi)
    cells = list(zip(*np.nonzero(mask_a != mask_b)))
    ok = True
    for c in cells:
        s = np.atleast_1d(cell_sum2(n, *c) if nd == 2 else cell_sums3(n, *c))
        if np.abs(s - accept).min() >= margin:
            ok = False
    return len(cells), ok


def num_cores2_ascending(N, offsets):
    """s_run.cpp:101-109 over a list in ascending offset order."""
    offs = np.sort(np.asarray(offsets, dtype=np.int64))
    dx = np.diff(offs % N)
    dy = np.diff(offs // N)
    pairs = np.count_nonzero((dy == 0) & (dx == 1)) + np.count_nonzero((dy == 1) & (dx == 0))
    return len(offs) - int(pairs)
