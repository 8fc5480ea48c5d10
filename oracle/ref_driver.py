"""CUDA driver-API wrapper that runs the reference's own device code.

TEST INFRASTRUCTURE ONLY (fixture generation and the reference-build
baseline).  `make ref` compiles harness TUs under oracle/ref_harness/, each
of which includes one of the reference's source files unchanged, into
cubins under oracle/_ref/.  This module loads those cubins through
libcuda.so.1 with ctypes -- no PyTorch, no code of the product -- so the
reference runs exactly as its own sources define it.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import byref, c_float, c_int, c_uint, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def have_cubin(name: str) -> bool:
    return os.path.exists(os.path.join(REF_DIR, name))


def D(p):
    """Mark an integer as a 64-bit device pointer kernel argument."""
    return ("u64", p)


class Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._ck(self.cu.cuInit(0), "cuInit")
        dev = c_int()
        self._ck(self.cu.cuDeviceGet(byref(dev), 0), "cuDeviceGet")
        ctx = c_void_p()
        self._ck(self.cu.cuDevicePrimaryCtxRetain(byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        self._ck(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        self.allocs = []

    @staticmethod
    def _ck(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def module(self, name):
        m = c_void_p()
        self._ck(self.cu.cuModuleLoad(byref(m), os.path.join(REF_DIR, name).encode()), "cuModuleLoad " + name)
        return m

    def fn(self, mod, name):
        f = c_void_p()
        self._ck(self.cu.cuModuleGetFunction(byref(f), mod, name.encode()), "cuModuleGetFunction " + name)
        return f

    def global_ptr(self, mod, name):
        p, n = c_uint64(), ctypes.c_size_t()
        self._ck(self.cu.cuModuleGetGlobal_v2(byref(p), byref(n), mod, name.encode()), "cuModuleGetGlobal " + name)
        return p.value

    def alloc(self, nbytes):
        p = c_uint64()
        self._ck(self.cu.cuMemAlloc_v2(byref(p), ctypes.c_size_t(max(nbytes, 4))), "cuMemAlloc")
        self.allocs.append(p.value)
        return p.value

    def memset8(self, dptr, value, nbytes):
        self._ck(self.cu.cuMemsetD8Async(c_uint64(dptr), ctypes.c_ubyte(value), ctypes.c_size_t(nbytes), None),
                 "cuMemsetD8Async")

    def h2d(self, dptr, arr):
        arr = np.ascontiguousarray(arr)
        self._ck(self.cu.cuMemcpyHtoD_v2(c_uint64(dptr), arr.ctypes.data_as(c_void_p),
                                         ctypes.c_size_t(arr.nbytes)), "cuMemcpyHtoD")

    def d2h(self, arr, dptr):
        self._ck(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data_as(c_void_p), c_uint64(dptr),
                                         ctypes.c_size_t(arr.nbytes)), "cuMemcpyDtoH")
        return arr

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        d = self.alloc(arr.nbytes)
        self.h2d(d, arr)
        return d

    @staticmethod
    def _params(args):
        vals = []
        for a in args:
            if isinstance(a, tuple):  # ('u64', value) device pointer
                vals.append(c_uint64(a[1]))
            elif isinstance(a, np.uint32):
                vals.append(c_uint(int(a)))
            else:
                vals.append(c_int(int(a)))
        return vals, (c_void_p * len(vals))(*[ctypes.cast(byref(v), c_void_p) for v in vals])

    def launch_async(self, f, grid, block, *args):
        vals, params = self._params(args)
        self._ck(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, None, params, None), "cuLaunchKernel")
        del vals

    def launch(self, f, grid, block, *args):
        self.launch_async(f, grid, block, *args)
        self.sync()

    def sync(self):
        self._ck(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def event(self):
        e = c_void_p()
        self._ck(self.cu.cuEventCreate(byref(e), 0), "cuEventCreate")
        return e

    def record(self, e):
        self._ck(self.cu.cuEventRecord(e, None), "cuEventRecord")

    def elapsed_ms(self, e0, e1):
        ms = c_float()
        self._ck(self.cu.cuEventElapsedTime(byref(ms), e0, e1), "cuEventElapsedTime")
        return float(ms.value)

    def destroy_event(self, e):
        self.cu.cuEventDestroy_v2(e)

    def free_all(self):
        for p in self.allocs:
            self.cu.cuMemFree_v2(c_uint64(p))
        self.allocs = []
