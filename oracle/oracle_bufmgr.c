/* oracle_bufmgr.c -- clock buffer-manager replay (TEST INFRASTRUCTURE ONLY). */
#include "pbm_oracle.h"
