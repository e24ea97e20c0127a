"""The C ABI library loads without a GPU and exports every entry point that
include/axs.h declares (no compute calls here)."""
import ctypes
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "axion-strings_gb300")


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "axs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(axs_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for must in ["axs_create", "axs_evolve", "axs_find_strings", "axs_powerspec", "axs_init_gaussian_thermal",
                 "axs_background", "axs_ensemble_evolve", "axs_upload", "axs_download"]:
        assert must in syms


def test_library_exports_every_declared_symbol():
    lib = os.path.join(PKG, "libaxs.so")
    if not os.path.exists(lib):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    h = ctypes.CDLL(lib)
    missing = [s for s in declared_symbols() if not hasattr(h, s)]
    assert not missing, missing


def test_python_mirror_covers_the_abi():
    src = open(os.path.join(PKG, "axs.py")).read()
    missing = [s for s in declared_symbols() if s not in src]
    assert not missing, missing
