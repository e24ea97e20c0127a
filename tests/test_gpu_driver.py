"""axs_run (the reference's main + run_standard on the C ABI) writes the
reference's output files. Their contents equal (a) the same sequence driven
through the ABI directly and (b) the files the reference's own program wrote
for the same parameter file (fixtures from oracle/_ref/ref_main)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from run_compare import RUNS, PRINT_UNIT, cmp_files, cmp_time_series, load_run

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "axion-strings_gb300")
DRIVER = os.path.join(PKG, "host", "axs_run")

PARAM = """% test run
lambda              1.0
enable_PRS          1
T_initial           4.0
NDIMS               {nd}
N                   {N}
space_step          0.5
time_step           0.1
stencil_setting     0
seed                77
write_output_file   1
output_file_path    {out}/output.txt
save_snapshots      1
n_snapshots         3
output_directory    {out}
save_fields         1
save_strings        1
save_pk             1
sample_time_series  1
n_samples           5
ts_output_path      {out}/time-series.csv
sample_strings      1
sample_background   1
thr                 1
enable_amr          0
init_from_snapshot  0
tau_initial         1.0
refinement_threshold 20.0
gpu_precision       64
final_step          {final}
"""


def every(t, n, final):
    period = final // (n - 1)
    return t == 0 or (period > 0 and t % period == 0)


def _driver():
    if not os.path.exists(DRIVER):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    return DRIVER


@pytest.mark.parametrize("nd,N,final", [(2, 64, 60), (3, 32, 40)])
def test_driver_outputs_match_abi(axs, tmp_path, nd, N, final):
    f = tmp_path / "run.param"
    f.write_text(PARAM.format(nd=nd, N=N, out=tmp_path, final=final))
    r = subprocess.run([_driver(), str(f)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    log = (tmp_path / "output.txt").read_text()
    assert "Running with" in log and "Time taken:" in log
    ts = (tmp_path / "time-series.csv").read_text().splitlines()
    assert ts[0] == "time,scalefactor,xi,n_plaquettes,phi1_bar,phi2_bar,phidot1_bar,phidot2_bar,axion_bar,saxion_bar"
    sample_steps = [t for t in range(final) if every(t, 5, final)]
    assert len(ts) - 1 == len(sample_steps)
    snap_steps = [t for t in range(final) if every(t, 3, final)]
    timings = (tmp_path / "snapshot-timings.csv").read_text().splitlines()
    assert timings[0] == "snapshot,tau,hubble_scale,string_tension,"
    assert len(timings) - 1 == len(snap_steps)

    # replay through the ABI
    p = axs.default_params(NDIMS=nd, N=N, lambda_=1.0, T_initial=4.0, space_step=0.5, time_step=0.1, seed=77,
                           precision=64, prs=1, thr=1)
    with axs.Lattice(p) as L:
        L.init_thermal(77)
        t = 0
        row = 1
        snap = 0
        for target in sorted(set(sample_steps + snap_steps)):
            L.evolve(target - t)
            t = target
            tau, _ = L.time
            if target in sample_steps:
                n, c, _ = L.find_strings()
                cols = ts[row].split(",")
                assert float(cols[0]) == pytest.approx(float("%f" % np.float32(0.5 * tau * tau)), abs=1e-6)
                assert int(cols[3]) == n
                assert cols[2] == "%f" % axs.xi(p, n, c, tau)
                bg = L.background()
                for q in range(6):
                    assert cols[4 + q] == "%f" % bg[q]
                row += 1
            if target in snap_steps:
                phi = L.download()
                raw = np.fromfile(tmp_path / ("snapshot%d-phi1" % snap), dtype=np.float64)
                want = phi[0].reshape(-1)[: raw.size]
                assert np.array_equal(raw, want)
                L.find_strings()
                pos = L.string_positions()
                lines = (tmp_path / ("snapshot%d-strings.csv" % snap)).read_text().splitlines()
                assert len(lines) == len(pos)
                if len(pos):
                    assert lines[0] == ", ".join(str(v) for v in pos[0])
                pk, ks, cnt = L.powerspec(axs.PHI2)
                pkl = (tmp_path / ("snapshot%d-pk.csv" % snap)).read_text().splitlines()
                assert pkl[0] == "k,pk,n_modes"
                ok = np.flatnonzero(cnt)
                assert len(pkl) - 1 == len(ok)
                first = ok[0]
                assert pkl[1] == "%e,%e,%d" % (ks[first], pk[first], cnt[first])
                snap += 1


# ---- against the reference's own program --------------------------------------

def _run_driver(text, out, extra=""):
    f = out / "run.param"
    f.write_text(text.format(out=out) + extra)
    r = subprocess.run([_driver(), str(f)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    return {p.name: p.read_bytes() for p in out.iterdir() if p.name not in ("run.param", "output.txt", "restart.ckpt")}


def _restart_from_reference_start(axs, out, nd, N, seed, off):
    """A checkpoint of the reference's initial state: gaussian_thermal on the
    device (the same deviates) plus the constant phidot offset of init.cpp's
    unset 3D k = 0 amplitude_dot, in the state a fresh run starts from."""
    p = axs.default_params(NDIMS=nd, N=N, lambda_=1.0, T_initial=4.0, space_step=0.5, time_step=0.1, seed=seed,
                           precision=64, prs=1, thr=1)
    with axs.Lattice(p) as L:
        L.init_thermal(seed)
        f = list(L.download())
        f[2] = f[2] + off[0]
        f[3] = f[3] + off[1]
        L.upload(*f)
        ck = L.checkpoint()
    path = out / "restart.ckpt"
    ck.tofile(str(path))
    return path


@pytest.mark.parametrize("name", RUNS)
def test_driver_matches_reference_run(axs, tmp_path, name):
    """axs_run on the reference's parameter file writes the files the
    reference's own main/run_standard wrote: same names, headers and row
    counts; time series and snapshot timings at the printed precision;
    spectra at the printed 7 digits; string lists equal (a cell within an ulp
    of atan2 of the threshold may differ, reported); raw field dumps within
    1e-10. In 3D the reference's phidot carries a constant offset from its
    unset k = 0 amplitude_dot (init.cpp:163-164), so the run there starts from
    that exact state (gpu_restart_file); a second run from the device's own
    gaussian_thermal must still agree at step 0 in everything but the two
    phidot means, which differ by that offset."""
    text, nd, N, seed, off, want = load_run(name)
    if nd == 2:
        got = _run_driver(text, tmp_path)
        assert sorted(got) == sorted(want)
        report = cmp_files(got, want, sorted(want))
    else:
        a = tmp_path / "from_reference_start"
        a.mkdir()
        ck = _restart_from_reference_start(axs, a, nd, N, seed, off)
        got = _run_driver(text, a, "gpu_restart_file %s\n" % ck)
        assert sorted(got) == sorted(want)
        report = cmp_files(got, want, sorted(want))
        b = tmp_path / "own_start"
        b.mkdir()
        own = _run_driver(text, b)
        assert sorted(own) == sorted(want)
        cmp_files(own, want, [f for f in want if f.startswith("snapshot0-")] + ["snapshot-timings.csv"])
        cmp_time_series(own["time-series.csv"], want["time-series.csv"], rows=[1],
                        skip=("phidot1_bar", "phidot2_bar"))
        g1 = own["time-series.csv"].decode().splitlines()[1].split(",")
        w1 = want["time-series.csv"].decode().splitlines()[1].split(",")
        for c, o in ((6, off[0]), (7, off[1])):
            assert abs(float(g1[c]) + o - float(w1[c])) <= 1.5 * PRINT_UNIT, (c, g1[c], w1[c], o)
    print(name, report)


def test_driver_checkpoint_resume_continues_run(axs, tmp_path):
    """gpu_checkpoint_file at the end of a run and gpu_restart_file at the
    start of the next: a run stopped at step 40 and resumed to step 60 writes
    the rows of steps 40.. that one run to 60 writes, and ends in the same
    state."""
    text = PARAM.format(nd=3, N=32, out="{out}", final="{final}")
    whole, first, second = (tmp_path / d for d in ("whole", "first", "second"))
    for d in (whole, first, second):
        d.mkdir()
    ck1 = first / "end.ckpt"
    ck2 = second / "end.ckpt"
    ckw = whole / "end.ckpt"
    _run_driver(text.replace("{final}", "60"), whole, "gpu_checkpoint_file %s\n" % ckw)
    _run_driver(text.replace("{final}", "40"), first, "gpu_checkpoint_file %s\n" % ck1)
    # the resumed run keeps the 60-step cadence (samples every 15 steps)
    _run_driver(text.replace("{final}", "60"), second,
                "gpu_restart_file %s\ngpu_checkpoint_file %s\n" % (ck1, ck2))
    assert ck2.read_bytes() == ckw.read_bytes()
    w = (whole / "time-series.csv").read_text().splitlines()
    s = (second / "time-series.csv").read_text().splitlines()
    assert s[0] == w[0]
    assert s[1:] == [r for r, t in zip(w[1:], range(0, 60, 15)) if t >= 40]
