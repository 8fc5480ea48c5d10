/* oracle_malloc.c -- size-classed malloc replay (TEST INFRASTRUCTURE ONLY). */
#include "pbm_oracle.h"
