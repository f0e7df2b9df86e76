/* Stub for building the reference's BLAZE_gpu sources as the oracle's
 * cross-check (test infrastructure only): gpu_cpu_common.h includes this NCBI
 * header. The only things the reference's code takes from it (through NCBI's
 * ncbi_std.h) are the MIN and MAX macros. */
#pragma once
#ifndef MAX
#define MAX(a, b) ((a) >= (b) ? (a) : (b))
#endif
#ifndef MIN
#define MIN(a, b) ((a) <= (b) ? (a) : (b))
#endif
