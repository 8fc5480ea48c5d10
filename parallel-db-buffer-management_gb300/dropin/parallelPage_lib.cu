// parallelPage_lib.cu -- the -rdc link form of the parallelPage.cuh drop-in.
//
// Compiled once with -rdc=true into libpbm_dropin.a.  A caller that defines
// PBM_PARALLELPAGE_RDC before including pbm/parallelPage.cuh sees only the
// declarations (extern, as source/parallelPage.cuh:7-75 declares them) and
// links this library, so all of its translation units share one set of
// free-page maps and one page store, as callers of the reference's
// separately compiled parallelPage.cu do (README.md:7-13).  Build it with the
// caller's TOTAL_N_PAGES and PAGE_SIZE when they differ from the defaults.
#define PBM_PARALLELPAGE_LIBRARY
#include "pbm/parallelPage.cuh"
