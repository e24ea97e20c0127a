"""The oracle pinned at the level of the whole run: run_standard
(src/standard/s_run.cpp:26-232) replayed on the oracle's functions writes the
files that the reference's own program wrote for the same parameter file
(fixtures tests/golden/run_*.npz from oracle/_ref/ref_main), compared as the
GPU driver's files are. CPU only; the 3D 256^3 run is left to the GPU test
(636 oracle steps of 16.8M sites take minutes on a CPU)."""
import math

import numpy as np
import pytest

import oracle_lib
from run_compare import cmp_files, load_run, param_value

f32 = np.float32


def _c_round(x):
    """C's round() for the positive values of s_run.cpp:82."""
    return math.floor(float(x) + 0.5)


def _every(t, n, final, enabled):   # s_run.cpp:14-24
    if not enabled:
        return False
    period = final // (n - 1)
    return t == 0 or (period > 0 and t % period == 0)


def oracle_run(orc, text, nd, N, seed, off):
    """Output files of run_standard with the oracle's step, finder, spectrum
    and background means, in the formats of fileio.cpp and s_run.cpp."""
    iv = lambda tag: int(param_value(text, tag))
    p = oracle_lib.make_params(NDIMS=nd, N=N, lam=1.0, T0=float(param_value(text, "T_initial")), dx=0.5, dt=0.1,
                               thr=iv("thr"), prs=1)
    f = list(orc.init_thermal(p, seed))
    f[2] = f[2] + off[0]
    f[3] = f[3] + off[1]
    dt, dx = f32(0.1), f32(0.5)
    lct = f32(0.5) * f32(N) * dx                          # physics.cpp:29
    final = _c_round(f32(lct / dt)) - _c_round(f32(dx / dt)) + 1
    samples, snaps = iv("n_samples"), iv("n_snapshots")
    ts = ["time,scalefactor,xi,n_plaquettes,phi1_bar,phi2_bar,phidot1_bar,phidot2_bar,axion_bar,saxion_bar"]
    timings = ["snapshot,tau,hubble_scale,string_tension,"]
    files = {}
    tau, ker, t = 1.0, None, 0
    nsnap = 0
    for target in range(final):
        sample = _every(target, samples, final, iv("sample_time_series"))
        snap = _every(target, snaps, final, iv("save_snapshots"))
        if not (sample or snap):
            continue
        if target > t:
            *f, tau, ker = orc.evolve(p, *f[:4], target - t, tau=tau, ker=ker, return_ker=True)
            t = target
        theta = np.arctan2(f[0], f[1])
        if sample:
            n, mask = orc.cores(p, theta)
            cores = orc.num_cores2(N, mask) if nd == 2 else n
            row = "%f,%f" % (f32(0.5 * tau * tau), f32(tau))
            row += ",%f,%d" % (orc.xi(p, n, cores, tau), n)
            row += "".join(",%f" % v for v in orc.background(p, *f[:4]))
            ts.append(row)
        if snap:
            h = f32(1.0 / (tau * tau))                     # physics.cpp:57-59
            tension = np.log(f32(1.0) / h)                  # physics.cpp:71-73 (float log)
            timings.append("%d,%f,%f,%f," % (nsnap, tau, f32(f32(1.0) / h), tension))
            if iv("save_fields"):
                cnt = N * N
                files["snapshot%d-phi1" % nsnap] = f[0].reshape(-1)[:cnt].tobytes()
                files["snapshot%d-phi2" % nsnap] = f[1].reshape(-1)[:cnt].tobytes()
            if iv("save_strings"):
                _, mask = orc.cores(p, theta)
                offs = np.flatnonzero(mask.reshape(-1))
                if nd == 2:
                    lines = ["%d, %d" % (m % N, m // N) for m in offs]
                else:
                    lines = ["%d, %d, %d" % (m // (N * N), (m // N) % N, m % N) for m in offs]
                files["snapshot%d-strings.csv" % nsnap] = "".join(x + "\n" for x in lines).encode()
            if iv("save_pk"):
                pk, ks, c = orc.powerspec(p, f[1])
                rows = ["k,pk,n_modes"] + ["%e,%e,%d" % (ks[b], pk[b], c[b]) for b in range(len(c)) if c[b] != 0]
                files["snapshot%d-pk.csv" % nsnap] = "".join(x + "\n" for x in rows).encode()
            nsnap += 1
    files["time-series.csv"] = "".join(x + "\n" for x in ts).encode()
    files["snapshot-timings.csv"] = "".join(x + "\n" for x in timings).encode()
    return files


@pytest.mark.parametrize("name", ["run_2d64", "run_3d24", "run_2d512"])
def test_oracle_run_matches_reference_run(oracle, name):
    text, nd, N, seed, off, want = load_run(name)
    got = oracle_run(oracle, text, nd, N, seed, off)
    assert sorted(got) == sorted(want)
    print(name, cmp_files(got, want, sorted(want)))
