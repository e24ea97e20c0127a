"""The axs_run driver's parameter-file reader keeps the reference's rules and
messages (src/common/read_parameters.cpp:182-238). CPU only: parsing happens
before any device call."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "axion-strings_gb300")
DRIVER = os.path.join(PKG, "host", "axs_run")

REFERENCE_TAGS = """
lambda              1.0
enable_PRS          1
T_initial           4.0
NDIMS               2
N                   64
space_step          0.5
time_step           0.1
stencil_setting     0
seed                1998
write_output_file   0
output_file_path    {out}/output.txt
save_snapshots      0
n_snapshots         5
output_directory    {out}
save_fields         0
save_strings        0
save_pk             0
sample_time_series  0
n_samples           40
ts_output_path      {out}/time-series.csv
sample_strings      0
sample_background   0
thr                 1
enable_amr          0
init_from_snapshot  0
tau_initial         1.0
refinement_threshold 20.0
"""


@pytest.fixture(scope="module")
def driver():
    if not os.path.exists(DRIVER):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    return DRIVER


def run(driver, text, tmp_path):
    f = tmp_path / "p.param"
    f.write_text(text.format(out=tmp_path))
    r = subprocess.run([driver, str(f)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    return r, str(f)


def test_usage(driver):
    r = subprocess.run([driver], stdout=subprocess.PIPE, text=True)
    assert r.returncode != 0 and "usage" in r.stdout


def test_missing_tag_message(driver, tmp_path):
    text = "\n".join(l for l in REFERENCE_TAGS.splitlines() if not l.startswith("lambda"))
    r, f = run(driver, text, tmp_path)
    assert r.returncode != 0
    assert "Error. I miss a value for tag 'lambda' in parameter file '%s'." % f in r.stdout


def test_duplicate_tag_message(driver, tmp_path):
    r, f = run(driver, REFERENCE_TAGS + "N 32\n", tmp_path)
    assert r.returncode != 0
    assert "Error in file %s:   Tag 'N' not allowed or multiple defined." % f in r.stdout


def test_unknown_tag_message(driver, tmp_path):
    r, f = run(driver, REFERENCE_TAGS + "bogus 1\n", tmp_path)
    assert "Tag 'bogus' not allowed or multiple defined." in r.stdout


def test_comments_and_gpu_tags_are_accepted(driver, tmp_path):
    text = "% a comment line\n" + REFERENCE_TAGS + "gpu_precision 32\ngpu_prs 1\nfinal_step 0\n"
    r, f = run(driver, text, tmp_path)
    # parsing succeeds: the run starts (and on a machine without a GPU fails in axs_create)
    assert "Running with" in r.stdout
    assert "not allowed" not in r.stdout and "I miss a value" not in r.stdout


def test_reference_default_param_parses(driver, tmp_path):
    import oracle_lib
    checkout = oracle_lib.reference_checkout()
    if checkout is None:
        pytest.skip("reference checkout not present (set AXS_REFERENCE_DIR)")
    ref = os.path.join(checkout, "default.param")
    r = subprocess.run([driver, ref], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert "not allowed" not in r.stdout and "I miss a value" not in r.stdout
