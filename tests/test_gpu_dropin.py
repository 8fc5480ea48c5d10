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


def test_rwmalloc_dropin_blocks_are_private_and_released(cuda, pbm_mod):
    """mallocRW / freeRW from a caller's kernels: every block is filled with
    its owner's id and read back intact (no overlap), and freeRW of every
    block returns the pool to its starting occupancy."""
    import numpy as np

    os.makedirs(BUILD, exist_ok=True)
    out_so = os.path.join(BUILD, "libcaller_RWMalloc.so")
    libdir = os.path.join(PKG, "lib")
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", '-DPBM_FAMILY_HEADER="pbm/RWMalloc.cuh"',
           "-DPBM_WITH_MALLOC", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "caller", "dropin_caller.cu"), "-o", out_so,
           "-L", libdir, "-lpbm", "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lib = ctypes.CDLL(out_so)
    n = 3000
    sizes = np.clip(np.exp(np.random.default_rng(4).uniform(np.log(16), np.log(65536), n)), 16, 65536)
    sizes = (sizes.astype(np.int32) // 4) * 4
    out = (ctypes.c_longlong * 4)()
    rc = lib.dropin_malloc_run(1, 4096, n, sizes.ctypes.data_as(ctypes.c_void_p), out)
    assert rc == 0
    bad, f0, f1, f2 = list(out)
    assert bad == 0
    assert f0 == 1_000_000 and f1 < f0
    assert f2 == f0


@pytest.fixture(scope="module")
def pp_caller(pbm_mod):
    os.makedirs(BUILD, exist_ok=True)
    out_so = os.path.join(BUILD, "libcaller_parallelPage.so")
    libdir = os.path.join(PKG, "lib")
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "caller", "pp_caller.cu"), "-o", out_so,
           "-L", libdir, "-lpbm", "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ctypes.CDLL(out_so)


def _build_so(name, sources, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    out_so = os.path.join(BUILD, name)
    libdir = os.path.join(PKG, "lib")
    cmd = (["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
            "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include")] + list(extra)
           + [os.path.join(ROOT, "tests", "caller", s) for s in sources]
           + ["-o", out_so, "-L", libdir] + (["-lpbm_dropin"] if "-rdc=true" in extra else [])
           + ["-lpbm", "-Xlinker", "-rpath", "-Xlinker", libdir])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ctypes.CDLL(out_so)


def test_parallel_page_strategies_share_one_page_store(cuda, pbm_mod):
    """pageAddress names the same page memory for all nine strategies: a
    payload written for the first strategy's page survives initialising the
    other eight, which add their maps but no second page store."""
    lib = _build_so("libcaller_pp_store.so", ["pp_caller.cu"])
    out = (ctypes.c_longlong * 3)()
    assert lib.pp_shared_store(out) == 0
    took, payload, store = list(out)
    assert payload == 0x5A5A1234
    # their maps (three with 2^22 per-thread slots) are far below one more store, let alone eight
    assert took < store


def test_parallel_page_rdc_two_units_share_one_pool(cuda, pbm_mod):
    """The -rdc link form (libpbm_dropin.a, README.md:7-13 of the reference):
    one translation unit takes pages, another checks their payloads and frees
    them, and the shared map's free count returns to its start."""
    import numpy as np

    lib = _build_so("libcaller_rdc.so", ["pp_rdc_alloc.cu", "pp_rdc_free.cu"], ["-rdc=true"])
    n = 20000
    ids = np.zeros(n, dtype=np.int32)
    out = (ctypes.c_longlong * 4)()
    assert lib.rdc_run(n, ids.ctypes.data_as(ctypes.c_void_p), out) == 0
    bad, f0, f1, f2 = list(out)
    assert bad == 0
    assert (ids >= 0).all() and np.unique(ids).size == n and (ids < 41_900_000).all()
    assert f0 == 41_900_000 and f0 - f1 == n and f2 == f0


@pytest.mark.parametrize("which", list(range(12)))
def test_parallel_page_dropin(cuda, pp_caller, which):
    """Every strategy of the monolithic API, called from a caller's kernel:
    unique in-range pages (runs of X pages for getXPage*), payloads intact,
    frees give the pages back."""
    import numpy as np

    n = 20000
    ids = np.zeros(n, dtype=np.int32)
    out = (ctypes.c_longlong * 4)()
    rc = pp_caller.pp_run(which, n, ids.ctypes.data_as(ctypes.c_void_p), out)
    assert rc == 0
    bad, f0, f1, f2 = list(out)
    assert bad == 0
    x = {9: 4, 10: 3, 11: 2}.get(which, 1)
    assert (ids >= 0).all() and (ids + x <= 1000000).all()
    cover = np.zeros(1000000, dtype=np.int32)
    for k in range(x):
        np.add.at(cover, ids + k, 1)
    assert cover.max() == 1
    assert f0 - f1 == n * x
    if which <= 8:
        assert f2 == f0


@pytest.mark.parametrize("which", [0, 1])
def test_malloc_classes_dropin(cuda, pbm_mod, which):
    """KernelMallocSimple / KernelMallocCollab passed by value into a caller's
    kernels (unitTestMalloc1.cu shape): blocks hold their owner's bytes and
    free() gives every page back."""
    os.makedirs(BUILD, exist_ok=True)
    out_so = os.path.join(BUILD, "libcaller_malloc.so")
    if not os.path.exists(out_so):
        libdir = os.path.join(PKG, "lib")
        cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17",
               "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "caller", "malloc_caller.cu"), "-o", out_so,
               "-L", libdir, "-lpbm", "-Xlinker", "-rpath", "-Xlinker", libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
    lib = ctypes.CDLL(out_so)
    out = (ctypes.c_longlong * 4)()
    assert lib.malloc_run(which, 20000, out) == 0
    bad, f0, f1, f2 = list(out)
    assert bad == 0 and f1 < f0 and f2 == f0


def test_malloc_simple_bumps_through_a_chunk_per_thread(cuda, pbm_mod):
    """KernelMallocSimple is the reference's per-thread chunk allocator
    (malloc.cu:100-152): a thread's small mallocs are consecutive slices of
    its own chunk (one page per thread here), and freeing them plus retire()
    gives every page back."""
    lib = _build_so("libcaller_malloc_bump.so", ["malloc_caller.cu"])
    out = (ctypes.c_longlong * 4)()
    n = 20000
    assert lib.malloc_bump_run(n, out) == 0
    bad, f0, f1, f2 = list(out)
    assert bad == 0
    assert abs((f0 - f1) / 1e6 * (1 << 18) - n) < 2     # one page per thread
    assert f2 == f0
