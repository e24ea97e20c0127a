"""axs_run (the reference's main + run_standard on the C ABI) writes the
reference's output files; their contents equal the same sequence driven
through the ABI directly."""
import os
import subprocess
import sys

import numpy as np
import pytest

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


@pytest.mark.parametrize("nd,N,final", [(2, 64, 60), (3, 32, 40)])
def test_driver_outputs_match_abi(axs, tmp_path, nd, N, final):
    if not os.path.exists(DRIVER):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    f = tmp_path / "run.param"
    f.write_text(PARAM.format(nd=nd, N=N, out=tmp_path, final=final))
    r = subprocess.run([DRIVER, str(f)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
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
