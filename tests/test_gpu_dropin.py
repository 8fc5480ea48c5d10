"""A caller's kernels written against the reference's header-only device API
link unchanged against the drop-in headers (one family per translation unit,
as with the reference): get/free from the caller's own kernels, payloads
through pageAddress/getPageID, and the host helpers' occupancy numbers."""
import ctypes
import os
import subprocess

import pytest

from conftest import PKG, ROOT

pytestmark = pytest.mark.gpu

FAMILIES = ["RandomWalkBasic", "RandomWalkBasic_BM", "CollabRW_BM", "CRW_BM"]
BUILD = os.path.join(ROOT, "tests", "caller", "_build")


def _compile(family):
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, f"libcaller_{family}.so")
    src = os.path.join(ROOT, "tests", "caller", "dropin_caller.cu")
    libdir = os.path.join(PKG, "lib")
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a",
           f'-DPBM_FAMILY_HEADER="pbm/{family}.cuh"', "-I", os.path.join(ROOT, "include"),
           src, "-o", out, "-L", libdir, "-lpbm", "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.fixture(scope="module")
def callers(pbm_mod):
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(4) as ex:
        libs = dict(zip(FAMILIES, ex.map(_compile, FAMILIES)))
    return libs


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("n,block", [(20000, 32), (5003, 96)])
def test_reference_style_driver(cuda, callers, family, n, block):
    lib = ctypes.CDLL(callers[family])
    out = (ctypes.c_longlong * 7)()
    rc = lib.dropin_run(1, 4096, ctypes.c_float(0.5), n, block, out)
    assert rc == 0
    bad, f0, f1, f2, f3, T, ssum = list(out)
    assert T == (1 << 30) // 4096
    assert bad == 0                                    # every caller got a page and kept its payload
    assert abs(f0 / 1e6 - 0.5) < 1e-3                  # prefillBuffer(0.5)
    assert abs((f0 - f1) / 1e6 - n / T) < 2e-6         # n pages taken
    assert f2 == f0                                    # freed exactly those pages
    assert f3 == 1_000_000                             # resetMemoryManager()
    assert ssum >= n
