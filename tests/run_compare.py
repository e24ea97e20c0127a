"""Runs of the reference's own main/run_standard (fixtures tests/golden/run_*.npz,
made by tests/golden/make_golden.py from oracle/_ref/ref_main) and the
comparison of another run's output files with them, file by file.

Output formats are those of src/common/fileio.cpp and src/standard/s_run.cpp:
time-series.csv and snapshot-timings.csv print with "%f", power spectra with
"%e" (7 significant digits), string lists as "%d, %d[, %d]", fields as raw
doubles."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RUNS = ["run_2d64", "run_3d24", "run_2d512", "run_3d256"]
PRINT_UNIT = 1.0e-6   # one unit in the last place of "%f"


def load_run(name):
    """(parameter-file text with an {out} placeholder, NDIMS, N, seed,
    3D k = 0 phidot offsets, {file name: bytes})."""
    z = np.load(os.path.join(GOLD, name + ".npz"))
    files = {k[5:]: bytes(z[k]) for k in z.files if k.startswith("file:")}
    return (str(z["param"]), int(z["nd"]), int(z["N"]), int(z["seed"]),
            [float(v) for v in z["k0_phidot_offset"]], files)


def param_value(text, tag):
    for line in text.splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == tag:
            return parts[1]
    raise KeyError(tag)


def cmp_time_series(got, want, rows=None, skip=()):
    """Header byte-equal, same rows; n_plaquettes and xi equal; other columns
    equal at the printed precision (within one unit of the last printed
    digit, for values on a rounding boundary). Returns (cells compared, cells
    byte-equal)."""
    g, w = got.decode().splitlines(), want.decode().splitlines()
    assert g[0] == w[0]
    assert len(g) == len(w), (len(g), len(w))
    head = w[0].split(",")
    n = eq = 0
    for r in (range(1, len(w)) if rows is None else rows):
        a, b = g[r].split(","), w[r].split(",")
        assert len(a) == len(b)
        for c, (x, y) in enumerate(zip(a, b)):
            if head[c] in skip:
                continue
            n += 1
            eq += x == y
            if head[c] in ("n_plaquettes", "xi"):
                assert x == y, ("row", r, head[c], x, y)
            else:
                assert abs(float(x) - float(y)) <= 1.5 * PRINT_UNIT, ("row", r, head[c], x, y)
    return n, eq


def cmp_pk(got, want):
    """k,pk,n_modes rows: counts equal, values equal at the printed 7 digits."""
    g, w = got.decode().splitlines(), want.decode().splitlines()
    assert g[0] == w[0] == "k,pk,n_modes"
    assert len(g) == len(w)
    eq = 0
    for x, y in zip(g[1:], w[1:]):
        a, b = x.split(","), y.split(",")
        assert a[2] == b[2]
        for u, v in zip(a[:2], b[:2]):
            assert abs(float(u) - float(v)) <= 2e-6 * abs(float(v)), (x, y)
        eq += x == y
    return len(w) - 1, eq


def cmp_files(got, want, names, field_tol=1e-10):
    """Compare the named output files; returns a report {name: summary}."""
    report = {}
    for f in names:
        assert f in got, ("missing output", f)
        a, b = got[f], want[f]
        if f == "time-series.csv":
            report[f] = cmp_time_series(a, b)
        elif f == "snapshot-timings.csv":
            assert a == b, (f, a, b)
            report[f] = "byte-equal"
        elif f.endswith("-pk.csv"):
            report[f] = cmp_pk(a, b)
        elif f.endswith("-strings.csv"):
            la, lb = a.decode().splitlines(), b.decode().splitlines()
            diff = set(la) ^ set(lb)
            # ascending offsets on both sides (a serial reference run); a cell
            # may move only if an ulp of atan2 moves it across the threshold
            assert len(diff) <= 2, (f, sorted(diff)[:6])
            if not diff:
                assert la == lb, f
            report[f] = (len(lb), len(diff))
        else:   # raw data_t field dumps (fileio.cpp:15-46)
            x, y = np.frombuffer(a, np.float64), np.frombuffer(b, np.float64)
            assert x.size == y.size, f
            err = float(np.abs(x - y).max() / np.abs(y).max())
            assert err <= field_tol, (f, err)
            report[f] = err
    return report
