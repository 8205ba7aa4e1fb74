/*
 * Minimal stand-in for oneTBB's parallel_for header, written for this project.
 * TEST INFRASTRUCTURE: the reference includes it (mo_lradtopo_horayzon.cpp:14)
 * but only calls parallel_reduce; this header just pulls in the range type.
 */
#ifndef HZ_SHIM_TBB_PARALLEL_FOR_H
#define HZ_SHIM_TBB_PARALLEL_FOR_H
#include "blocked_range.h"
#endif
