// fx_common.cuh -- shared prelude of the reference harness TUs.
//
// TEST INFRASTRUCTURE ONLY.  Each h_*.cu includes one of the reference's
// own source files (from its source/ directory, via -I) after this prelude
// and adds extern "C" kernels that point the reference's __device__ globals
// at caller-supplied buffers and call its device routines one thread / one
// warp at a time.  The reference seeds its walks from clock(); the macro
// below replaces that read with a value the harness sets before each call,
// which makes single-thread and single-warp runs reproducible.  Nothing else
// in the reference's code is changed.
#pragma once
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include <time.h>
#include <assert.h>
#include <iostream>
#include <cub/cub.cuh>
#include <cooperative_groups.h>

__device__ int fx_clock_val;
#define clock() (fx_clock_val)

// global thread id of the caller (the reference's own tid expression)
__device__ __forceinline__ int fx_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }
