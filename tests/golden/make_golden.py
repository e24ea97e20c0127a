"""Generate the golden fixtures of tests/golden/ from the reference's own
hot-path sources, compiled from the reference tree against the project's
MKL/FFTW shims by `make -C oracle ref` (needs the reference checkout).

Fixtures (all small):
  fdm_matrix_n4.txt     the exact 16x16 matrix golden of src/tests/fdm_matrix.cpp:47-64
  strings_*.npz         theta snapshots and the reference's cores2/cores3 masks
  step_*.npz            thermal initial state and the reference's state after 1 / 10
                        vvsl_field_rescaled steps
  pk_*.npz              output_powerspec of a stepped field
  run_*.npz             every output file of the reference's own program
                        (src/main.cpp -> run_standard, oracle/_ref/ref_main) for a
                        parameter file: 2D 64^2 and 3D 24^3 with fields, strings and
                        spectra; 2D 512^2 and 3D 256^3 with the time series and spectra;
                        plus, in 3D, the constant phidot offset of init.cpp's unset
                        k = 0 amplitude_dot

The reference's random numbers come from the shim (Philox + Box-Muller), not
MKL, so the initial states pin the restatement of init.cpp's arithmetic, not
MKL's bitstream.

The reference checkout is $AXS_REFERENCE_DIR, or a folder named `reference`
beside this repository.

Usage: python tests/golden/make_golden.py [fixtures] [runs]  (from the repository root)
"""
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib  # noqa: E402
from strings_util import accept_value, near_threshold_theta, num_cores2_ascending  # noqa: E402

_CHECKOUT = oracle_lib.reference_checkout()   # $AXS_REFERENCE_DIR, or `reference` beside the repo
REF_SRC = os.path.join(_CHECKOUT, "src") if _CHECKOUT else ""


def fdm_matrix():
    text = open(os.path.join(REF_SRC, "tests", "fdm_matrix.cpp")).read()
    body = re.search(r"correct_matrix\[\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    assert len(vals) == 256
    np.savetxt(os.path.join(HERE, "fdm_matrix_n4.txt"), np.array(vals).reshape(16, 16), fmt="%d")


def strings(ref):
    rng = np.random.default_rng(20240601)
    for nd, N, thr in [(2, 64, 1), (3, 16, 1), (3, 16, 30)]:
        p = oracle_lib.make_params(NDIMS=nd, N=N, thr=thr)
        for kind in ("uniform", "near"):
            if kind == "uniform":
                theta = rng.uniform(-np.pi, np.pi, (N,) * nd)
            else:
                theta = near_threshold_theta(rng, nd, N, accept_value(thr))
            n, pos = ref.cores(p, theta)
            if nd == 2:
                offs = pos[:, 0] + N * pos[:, 1]
            else:
                offs = (pos[:, 0].astype(np.int64) * N + pos[:, 1]) * N + pos[:, 2]
            mask = np.zeros(theta.size, dtype=np.uint8)
            mask[offs] = 1
            extra = {}
            if nd == 2:
                extra["num_cores_serial"] = num_cores2_ascending(N, offs)
            np.savez_compressed(os.path.join(HERE, "strings_%dd%d_thr%d_%s.npz" % (nd, N, thr, kind)),
                                nd=nd, N=N, thr=thr, theta=theta, n=n, mask_bits=np.packbits(mask), **extra)


def steps(ref):
    for nd, N, seed, lam, T0 in [(2, 32, 5, 1.0, 4.0), (3, 16, 6, 1.0, 4.0)]:
        p = oracle_lib.make_params(NDIMS=nd, N=N, lam=lam, T0=T0, dx=0.5, dt=0.1)
        f0 = ref.gaussian_thermal(p, seed)
        f1 = ref.evolve(p, *f0, 1)
        f10 = ref.evolve(p, *f0, 10)
        np.savez_compressed(os.path.join(HERE, "step_%dd%d.npz" % (nd, N)), nd=nd, N=N, seed=seed, lam=lam, T0=T0,
                            dx=0.5, dt=0.1, s0=np.stack(f0), s1=np.stack(f1[:4]), s10=np.stack(f10[:4]),
                            tau1=f1[4], tau10=f10[4])
        pk, ks, cnt = ref.powerspec(p, f10[1])
        np.savez_compressed(os.path.join(HERE, "pk_%dd%d.npz" % (nd, N)), pk=pk, ks=ks, count=cnt)


# Parameter file of the reference's own runs (every tag of
# read_parameters.cpp:30-172 exactly once); {out} is the output folder.
RUN_PARAM = """% reference run for the run-loop fixtures
lambda              1.0
enable_PRS          1
T_initial           4.0
NDIMS               {nd}
N                   {N}
space_step          0.5
time_step           0.1
stencil_setting     0
seed                {seed}
write_output_file   1
output_file_path    {{out}}/output.txt
save_snapshots      1
n_snapshots         {snaps}
output_directory    {{out}}
save_fields         {fields}
save_strings        {strings}
save_pk             1
sample_time_series  1
n_samples           {samples}
ts_output_path      {{out}}/time-series.csv
sample_strings      1
sample_background   1
thr                 1
enable_amr          0
init_from_snapshot  0
tau_initial         1.0
refinement_threshold 20.0
"""

# (name, NDIMS, N, seed, n_snapshots, save_fields, save_strings, n_samples, threads):
# small full-output runs, and the 2D 512^2 and 3D 256^3 workloads with a
# plaquette count about every 100 and 20 steps (their strings and fields stay
# out: the files would be megabytes). 2D runs use one thread: the order of
# cores2's list is that of the OpenMP merge reduction (string_finding.cpp:10-12),
# ascending offsets only for a serial run, and the 2D core count
# (s_run.cpp:101-109) depends on it.
RUNS = [("run_2d64", 2, 64, 77, 3, 1, 1, 5, 1),
        ("run_3d24", 3, 24, 78, 3, 1, 1, 5, 1),
        ("run_2d512", 2, 512, 79, 5, 0, 0, 13, 1),
        ("run_3d256", 3, 256, 80, 3, 0, 0, 32, 0)]


def k0_phidot_offset(nd, N, seed):
    """init.cpp:151-171 leaves amplitude_dot unset at k = 0 in 3D
    (:163-164 assign amplitude twice); compiled as here it keeps the value of
    the loop's previous mode. The reference's phidot then differs from the
    restatement's (amplitude_dot = 0 there) by a constant per component:
    returned as (offset_phidot1, offset_phidot2), measured on the reference's
    own gaussian_thermal."""
    if nd == 2:
        return 0.0, 0.0
    ref = oracle_lib.load_ref(64)
    orc = oracle_lib.load()
    p = oracle_lib.make_params(NDIMS=nd, N=N, T0=4.0, dx=0.5, dt=0.1)

    class P:
        pass
    q = P()
    for k, v in dict(NDIMS=nd, N=N, lambda_=1.0, T_initial=4.0, space_step=0.5, time_step=0.1,
                     stencil_setting=0, thr=1).items():
        setattr(q, k, v)
    a = orc.init_thermal(p, seed)
    b = ref.gaussian_thermal(q, seed)
    out = []
    for c in (2, 3):
        d = b[c] - a[c]
        assert np.abs(d - d.mean()).max() <= 1e-12 * np.abs(a[c]).max(), "offset not constant"
        out.append(float(d.mean()))
    return tuple(out)


def runs():
    """The reference's own program (oracle/_ref/ref_main: main.cpp,
    read_parameter_file, fileio.cpp, run_standard) on small parameter files;
    every output file it writes, byte for byte."""
    import tempfile
    exe = os.path.join(oracle_lib.REF_DIR, "ref_main")
    for name, nd, N, seed, snaps, fields, strs, samples, threads in RUNS:
        text = RUN_PARAM.format(nd=nd, N=N, seed=seed, snaps=snaps, fields=fields, strings=strs, samples=samples)
        with tempfile.TemporaryDirectory(prefix="axs_") as out:
            pf = os.path.join(out, "run.param")
            with open(pf, "w") as fp:
                fp.write(text.format(out=out))
            env = dict(os.environ)
            if threads:
                env["OMP_NUM_THREADS"] = str(threads)
            subprocess.run([exe, pf], check=True, env=env, stdout=subprocess.DEVNULL)
            files = {}
            for f in sorted(os.listdir(out)):
                if f in ("run.param", "output.txt"):
                    continue
                files["file:" + f] = np.frombuffer(open(os.path.join(out, f), "rb").read(), dtype=np.uint8)
        off = k0_phidot_offset(nd, N, seed)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), param=text, nd=nd, N=N, seed=seed,
                            k0_phidot_offset=np.array(off), **files)
        print(name, len(files), "files")


def main():
    if not os.path.isdir(REF_SRC):
        raise SystemExit("reference sources not found: set AXS_REFERENCE_DIR to the reference checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF_SRC=" + REF_SRC], check=True)
    ref = oracle_lib.load_ref(64)
    only = sys.argv[1:]
    if not only or "fixtures" in only:
        fdm_matrix()
        strings(ref)
        steps(ref)
    if not only or "runs" in only:
        runs()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
