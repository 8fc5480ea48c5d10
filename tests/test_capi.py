"""The C-ABI library loads and exports every entry point include/pbm.h
declares (no device calls: runs without a GPU)."""
import ctypes
import os
import re

from conftest import PKG, ROOT


def header_functions():
    with open(os.path.join(ROOT, "include", "pbm.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pbm_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import pbm

    lib = ctypes.CDLL(pbm.LIB_PATH)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    import pbm

    bound = {n for n, _, _ in pbm.SIGNATURES}
    assert set(header_functions()) <= bound, set(header_functions()) - bound


def test_version_string_without_gpu():
    import pbm

    assert "sm_103a" in pbm.version()


def test_rdc_dropin_library_defines_the_host_api():
    """libpbm_dropin.a (the -rdc link form of parallelPage.cuh) defines every
    host function the header declares; the device functions travel as
    relocatable device code in the same objects."""
    import shutil
    import subprocess

    import pytest

    lib = os.path.join(PKG, "lib", "libpbm_dropin.a")
    assert os.path.exists(lib), "build() makes libpbm_dropin.a"
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-C", "--defined-only", lib], capture_output=True, text=True).stdout
    with open(os.path.join(ROOT, "include", "pbm", "parallelPage.cuh")) as f:
        hdr = f.read()
    host = sorted(set(re.findall(r"PBM_PP_API __host__ \w+(?: \w+)? (\w+)\(", hdr)))
    assert len(host) >= 25          # init, print and reset of the strategies, the monitor, pbmFreePagesLeft
    missing = [n for n in host if f" {n}(" not in out]
    assert not missing, missing
