// Drop-in for source/parallelPage.cuh + parallelPage.cu: the nine suffixed
// strategies of the monolithic API (names, signatures and defaults of
// parallelPage.cuh:7-75), each with its own free-page map of TOTAL_N_PAGES
// pages, all sharing one page store of TOTAL_N_PAGES x PAGE_SIZE bytes
// (parallelPage.cu:13-23, 53-71), so pageAddress means the same page for
// every strategy.  TOTAL_N_PAGES and PAGE_SIZE are compile-time, as in the
// reference (override the macros before including).
//
// Two ways to link, as with the reference (README.md:7-13):
//   header-only  include this header; each translation unit gets its own
//                maps and page store (the functions are inline);
//   -rdc         define PBM_PARALLELPAGE_RDC before including, compile with
//                -rdc=true and link libpbm_dropin.a (built with the same
//                TOTAL_N_PAGES and PAGE_SIZE, 41,900,000 x 264 by default) and
//                libpbm.so: the functions are the library's, so every
//                translation unit of the caller shares one set of maps and one
//                page store, as the reference's extern declarations imply.
// Every walk is bounded (PBM_DROPIN_MAX_STEPS) and returns -1 instead of
// trapping; int-per-page maps are bitmaps here.
#pragma once
#include <cstdint>
#include <cstdio>

#include <cuda_runtime.h>

#ifndef TOTAL_N_PAGES
#define TOTAL_N_PAGES 41900000
#endif
#ifndef PAGE_SIZE
#define PAGE_SIZE 264
#endif

#if defined(PBM_PARALLELPAGE_RDC) || defined(PBM_PARALLELPAGE_LIBRARY)
#define PBM_PP_API extern
#else
#define PBM_PP_API inline
#endif

/* pageAddress(pageID): parallelPage.cuh:7, parallelPage.cu:15-23 */
PBM_PP_API __device__ void* pageAddress(int pageID);

/* Random Walk: parallelPage.cuh:10-15 */
PBM_PP_API __host__ void initPagesRandomWalk();
PBM_PP_API __device__ int getPageRandomWalk(int* step_count = 0);
PBM_PP_API __device__ void freePageRandomWalk(int pageID);
PBM_PP_API __host__ void printNumPagesLeftRandomWalk();
PBM_PP_API __host__ void resetBufferRandomWalk();
PBM_PP_API __host__ void monitorBufferRandomWalk(int msGap = 100, int maxCount = 100);

/* Clustered Random Walk: parallelPage.cuh:20-23 */
PBM_PP_API __host__ void initPagesClusteredRandomWalk();
PBM_PP_API __device__ int getPageClusteredRandomWalk(int* step_count = 0);
PBM_PP_API __device__ void freePageClusteredRandomWalk(int pageID);
PBM_PP_API __host__ void printNumPagesLeftClusteredRandomWalk();

/* LinkedList: parallelPage.cuh:26-30 */
PBM_PP_API __host__ void initPagesLinkedList();
PBM_PP_API __device__ int getPageLinkedList(int* step_count = 0);
PBM_PP_API __device__ void freePageLinkedList(int pageID, int* step_count = 0);
PBM_PP_API __host__ void printNumPagesLeftLinkedList();
PBM_PP_API __host__ void resetBufferLinkedList();

/* Single Clock: parallelPage.cuh:33-37 */
PBM_PP_API __host__ void initPagesSingleClock();
PBM_PP_API __device__ int getPageSingleClock(int* step_count = 0);
PBM_PP_API __device__ void freePageSingleClock(int pageID, int* step_count = 0);
PBM_PP_API __host__ void printNumPagesLeftSingleClock();
PBM_PP_API __host__ void resetBufferSingleClock();

/* Distributed Clock: parallelPage.cuh:40-44 */
PBM_PP_API __host__ void initPagesDistClock();
PBM_PP_API __device__ int getPageDistClock(int* step_count = 0);
PBM_PP_API __device__ void freePageDistClock(int pageID, int* step_count = 0);
PBM_PP_API __host__ void printNumPagesLeftDistClock();
PBM_PP_API __host__ void resetBufferDistClock();

/* Collaborative Random Walk: parallelPage.cuh:47-51 */
PBM_PP_API __host__ void initPagesCollabRW();
PBM_PP_API __device__ int getPageCollabRW(int* step_count = 0);
PBM_PP_API __device__ void freePageCollabRW(int pageID);
PBM_PP_API __host__ void printNumPagesLeftCollabRW();
PBM_PP_API __host__ void resetBufferCollabRW();

/* Collaborative Random Walk + bitmap: parallelPage.cuh:54-59 */
PBM_PP_API __host__ void initPagesCollabRW_BM();
PBM_PP_API __device__ int getPageCollabRW_BM(int* step_count = 0);
PBM_PP_API __device__ int getXPageCollabRW_BM(int X, int* step_count = 0);
PBM_PP_API __device__ void freePageCollabRW_BM(int pageID);
PBM_PP_API __host__ void printNumPagesLeftCollabRW_BM();
PBM_PP_API __host__ void resetBufferCollabRW_BM();

/* Random Walk + bitmap: parallelPage.cuh:62-67 */
PBM_PP_API __host__ void initPagesRandomWalk_BM();
PBM_PP_API __device__ int getPageRandomWalk_BM(int* step_count = 0);
PBM_PP_API __device__ int getXPageRandomWalk_BM(int X, int* step_count = 0);
PBM_PP_API __device__ void freePageRandomWalk_BM(int pageID);
PBM_PP_API __host__ void printNumPagesLeftRandomWalk_BM();
PBM_PP_API __host__ void resetBufferRandomWalk_BM();

/* Clustered Random Walk + bitmap: parallelPage.cuh:70-75 */
PBM_PP_API __host__ void initPagesClusteredRandomWalk_BM();
PBM_PP_API __device__ int getPageClusteredRandomWalk_BM(int* step_count = 0);
PBM_PP_API __device__ int getXPageClusteredRandomWalk_BM(int X, int* step_count = 0);
PBM_PP_API __device__ void freePageClusteredRandomWalk_BM(int pageID);
PBM_PP_API __host__ void printNumPagesLeftClusteredRandomWalk_BM();
PBM_PP_API __host__ void resetBufferClusteredRandomWalk_BM();

/* No reference counterpart: the free pages of one strategy's map (its
 * index in the order above, 0 = RandomWalk .. 8 = ClusteredRandomWalk_BM;
 * 0 if it was never initialised), which printNumPagesLeft* print. */
PBM_PP_API __host__ unsigned long long pbmFreePagesLeft(int strategy);

/* gpuErrchk: parallelPage.cuh:79-86 (reports instead of exit()) */
#ifndef gpuErrchk
#define gpuErrchk(ans) pbm_gpu_report((ans), __FILE__, __LINE__)
inline void pbm_gpu_report(cudaError_t code, const char* file, int line) {
    if (code != cudaSuccess) std::fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
}
#endif

#ifndef PBM_PARALLELPAGE_RDC
#include "pbm/parallelPage_impl.cuh"
#endif
