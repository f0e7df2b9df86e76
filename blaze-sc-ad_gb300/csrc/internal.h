// internal.h -- calls between the library's own translation units that are
// not part of the C ABI.
#pragma once
#include <cstdint>
#include <new>

#include "blaze_prelim.h"

// Refills (creating it when *batch is null) a batch with new queries on the
// search context's stream, reusing its device buffers while they are large
// enough; validation and results as blaze_batch_create.
int batch_refill(blaze_search *s, blaze_batch **batch, const uint8_t *residues, const uint64_t *offsets,
                 uint32_t n_queries, int32_t word_threshold);

// The calling thread's last CUDA error (as a cudaError_t value), so that a
// worker thread's error can be handed to the thread that reads the status.
int last_cuda_error_code();
void set_last_cuda_error_code(int code);

// Handler of a function-try-block around a C entry point: no C++ exception
// (a failed host allocation or thread start) crosses the C ABI.
#define BLAZE_ABI_CATCH                                \
    catch (const std::bad_alloc &) {                   \
        return BLAZE_ERR_OUT_OF_MEMORY;                \
    }                                                  \
    catch (...) {                                      \
        return BLAZE_ERR_INTERNAL;                     \
    }
