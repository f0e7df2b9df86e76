// common.cuh -- internal types shared by the host driver and the kernels of
// libblaze103 (GB300 / sm_103a BLASTP preliminary stage).
#pragma once

#include <cstdint>
#include <climits>

#include <cuda_runtime.h>

#include "blaze_prelim.h"

namespace blaze {

constexpr int kAlphabet = 28;
constexpr int kWords = kAlphabet * kAlphabet * kAlphabet;  // 21952 three-letter words
constexpr int kWordSize = 3;
constexpr int32_t kNeg = INT32_MIN / 2;  // "minus infinity" of the gapped DP
constexpr int kWarp = 32;

// Word-finder tuning (per warp of the scan kernel).
constexpr int kDeferCap = 64;   // deferred hits per buffer (two buffers)
constexpr int kSeedCap = 64;    // queued two-hit seeds (>= kDeferCap)
constexpr int kScanMaxWarpsPerBlock = 32;
constexpr int kGappedWarpsPerBlock = 4;
constexpr int kPresenceWords = (kWords + 31) / 32;                     // 686
constexpr size_t kScanMatBytes = kAlphabet * kAlphabet;               // int8 matrix, 784
constexpr size_t kScanPresenceBytes = (kPresenceWords * 4 + 15) & ~15; // 2752
constexpr int32_t kQuerySmemMax = 8192;      // queries up to this length live in shared memory
constexpr uint32_t kScanStageBytes = 1024;   // subjects up to this length are staged
constexpr uint32_t kMaxTileResidues = 1u << 16;  // automatic tile size at most (residues per warp)

// An ungapped HSP that reached the ungapped cutoff (NCBI BlastInitHSP analog).
struct InitHit {
    int32_t q_start, s_start, len, score;
    int32_t q_trig, s_trig;  // the second word hit that triggered the extension
};

// One subject with init hits, for the gapped kernel.
struct WorkItem {
    uint32_t subject;  // index into the length-sorted database
    uint32_t n_init;
    uint64_t first;    // first record in the init-hit array
};

// One init hit's gapped extension for the lane-parallel DP: the subject, the
// query (batched: its index) and the gapped start point. Written by the prep
// kernel at the init hit's slot; valid = 0 for an init hit that is skipped.
struct DpTask {
    uint64_t s_base;  // offset of the subject's residues
    int32_t slen;
    uint32_t query;
    int32_t q_off, s_off;
    int32_t valid, pad;
};

// A finished gapped HSP as the device writes it (subject = sorted index).
struct DevHsp {
    uint32_t subject;
    int32_t score, q_start, q_end, s_start, s_end, q_gs, s_gs;
};

// Device counters of one run; zeroed before every run.
struct DevCounters {
    unsigned long long init_count;   // init hits published
    unsigned long long work_count;   // work items published
    unsigned long long out_count;    // HSPs published
    unsigned long long next_gapped;  // gapped-kernel work cursor
    unsigned long long word_hits;
    unsigned long long extensions;
    unsigned long long gapped_ext;
    unsigned long long dp_cells;
    unsigned long long residues;
    unsigned int overflow_subjects;  // subjects whose init hits exceeded the per-warp scratch
    unsigned int max_init_needed;    // largest init-hit count among those
    unsigned int flags;              // kFlag* bits
    unsigned int pad;
    unsigned long long group_count;  // subject HSP lists published (GroupDesc records)
    unsigned long long next_prep;    // gapped prep-kernel work cursor
    unsigned long long next_dp;      // lane DP task cursor
};

// One subject's HSP list in the gapped stage's output, after the preliminary
// E-value reap and max_hsps: `n` HSPs from `first`, best first. The hit-list
// selection sets n to 0 for a subject outside its query's hitlist_size.
struct GroupDesc {
    unsigned long long first;
    uint32_t query;    // batched runs: the query's position in its batch
    uint32_t subject;  // index into the length-sorted database
    uint32_t oid;
    uint32_t n;
    int32_t best;      // score of the list's first HSP
    uint32_t pad;
};

constexpr unsigned kFlagInitArrayFull = 1u;
constexpr unsigned kFlagWorkArrayFull = 2u;
constexpr unsigned kFlagOutArrayFull = 4u;
constexpr unsigned kFlagSavedFull = 8u;
constexpr unsigned kFlagBadState = 16u;
constexpr unsigned kFlagSubjectTooLong = 32u;  // gapped: a subject longer than its DP rows was skipped
constexpr unsigned kFlagBadInitHit = 64u;      // gapped: an init hit outside its query or subject was skipped

// One query of a batch, as the batched scan kernel reads it.
struct BatchQuery {
    const uint8_t *q;
    int32_t qlen;
    int32_t ungapped_cutoff;
    const uint32_t *cell_start, *cell_pack, *presence;
    const uint16_t *cell_off;
    uint32_t diag_entries, diag_magic;
    uint32_t index;  // position of the query in its batch
};

struct ScanArgs {
    const uint8_t *res;        // residues, length-sorted subjects
    const uint64_t *off;       // n_subj + 1 offsets
    uint32_t n_subj;
    const uint8_t *q;          // query residues
    int32_t qlen;
    const uint32_t *cell_start;  // kWords + 1
    const uint32_t *cell_pack;   // kWords: start << 8 | min(count, 255)
    const uint32_t *presence;    // kPresenceWords: bit w set when word w has hits
    const uint16_t *cell_off;    // query offsets per cell, ascending
    int32_t window, xdrop, cutoff;
    uint32_t diag_entries;       // >= qlen + window
    uint32_t diag_magic;         // floor(2^32 / diag_entries) + 1
    uint32_t diag_bytes, stage_bytes, query_smem_bytes, warp_smem_bytes;
    uint32_t diag_entries_max;   // largest table any query of the launch uses
    uint32_t smem_bytes;         // batched launches: dynamic shared memory of a block
    // batched launches only
    const BatchQuery *queries;   // n_queries descriptors
    uint32_t n_queries;
    const uint32_t *tile_bounds;  // n_ranges + 1 subject indices, descending: range r is [b[r+1], b[r])
    uint32_t n_ranges;
    uint32_t *work_query;        // query index of each work item (nullptr: one query)
    uint32_t query_index;        // single-query launches inside a batched pass: the query's index
    InitHit *scratch;          // per warp: scratch_cap records
    uint32_t scratch_cap;
    InitHit *init_out;
    unsigned long long init_cap;
    WorkItem *work;
    unsigned long long work_cap;
    DevCounters *cnt;
    unsigned long long *cursor;  // this launch's work cursor (zeroed before the pass)
};

struct GappedArgs {
    const uint8_t *res;
    const uint64_t *off;
    const uint8_t *q;
    int32_t qlen;
    // batched launches only: query of each work item and per-query data
    const uint32_t *work_query;
    const uint8_t *const *batch_q;
    const int32_t *batch_qlen;
    const int32_t *batch_cutoff;
    const int32_t *batch_smin;       // per query: lowest score the preliminary reap keeps
    const int32_t *batch_max_hsps;   // per query: HSPs kept per subject (0: all)
    const InitHit *init_in;
    const WorkItem *work;
    unsigned long long work_cap;
    unsigned long long init_cap;  // records in init_in (items beyond it are rejected)
    uint32_t n_subj, n_queries;   // valid subject and query indices of an item
    InitHit *sorted;     // per warp: cap records
    DevHsp *saved;       // per warp: cap records
    uint32_t cap;
    int32_t *dp;         // per warp: 2 * dp_stride ints, 8-byte aligned
    uint32_t dp_stride;  // >= max subject length + 2, even
    int32_t gap_open, gap_extend, xdrop, cutoff;
    int32_t smin, max_hsps;  // single query: as batch_smin / batch_max_hsps
    DevHsp *out;
    unsigned long long out_cap;
    const uint32_t *oid;     // sorted index -> OID
    GroupDesc *groups;       // one per published list (null: none written)
    uint32_t *qkept;         // per query: lists published (null: not counted)
    DevCounters *cnt;
    // the three-kernel form (launch_gapped_split), per init-hit slot
    InitHit *init_sorted;    // each item's init hits in processing order
    DpTask *dtask;
    int4 *dres;              // per slot: left and right DP (best, row, column, cells; cells -1: not run)
};

// Hit-list selection: queries that keep more subjects than their
// hitlist_size keep the hitlist_size best (score of the first HSP
// descending, ties by smaller OID); the others' lists are marked n = 0.
struct HitlistArgs {
    GroupDesc *groups;
    unsigned long long n_groups;
    const uint32_t *seg_off;         // per query: its segment of keys (n_queries + 1; empty if not selecting)
    uint32_t *seg_fill;              // per query: segment cursor, zeroed
    unsigned long long *keys;        // segment storage: ranking key and list index
    uint32_t *idx;
    const uint32_t *sel_queries;     // the selecting queries, one block each
    const int32_t *limit;            // per query: hitlist_size
};

// Shared-memory layout of the scan kernel for one query.
struct ScanLayout {
    uint32_t diag_entries, diag_magic, diag_bytes, stage_bytes, query_smem_bytes, warp_smem_bytes;
    int warps_per_block;
    size_t smem_bytes;
};

// Traceback stage: one preliminary HSP to trace from its gapped start point.
struct TbItem {
    uint32_t subject;  // index into the length-sorted database
    int32_t q_off, s_off;
    uint32_t query;    // batched runs: the query's position in its batch
};

struct TbOut {
    int32_t score, q_start, q_end, s_start, s_end;
    int32_t length, identities, positives, mismatches, gap_opens, gaps;
    int32_t status;  // 0 done, 1 direction buffer too small, 2 inconsistent path
    int32_t cells;   // DP cells computed (left and right)
};

struct TracebackArgs {
    const uint8_t *res;
    const uint64_t *off;
    const uint8_t *q;
    int32_t qlen;
    const uint8_t *const *batch_q;  // batched runs: per query (q, qlen unused)
    const int32_t *batch_qlen;
    const TbItem *items;
    uint32_t n_items;
    TbOut *out;
    int32_t gap_open, gap_extend, xdrop;
    int32_t *dp;                // per warp: H and E rows of dp_stride ints each
    uint32_t dp_stride;
    uint8_t *dirs;              // per warp: dir_cap direction bytes
    unsigned long long dir_cap;
    int32_t *rows;              // per warp: 3 ints (first, end, offset) per DP row
    uint32_t row_cap;
    unsigned long long *cursor;
};

// Launchers (scan.cu, kernels.cu, traceback.cu).
ScanLayout scan_layout(int32_t qlen, int32_t window, uint32_t stage_bytes, size_t smem_budget, int max_warps);
cudaError_t launch_scan(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem, cudaStream_t st);
cudaError_t scan_occupancy(bool query_in_smem, int warps_per_block, size_t smem, int *blocks_per_sm);
int scan_max_warps_by_registers(bool query_in_smem);
cudaError_t launch_gapped(const GappedArgs &a, int n_blocks, cudaStream_t st,
                          int warps_per_block = kGappedWarpsPerBlock);
cudaError_t launch_hitlist(const HitlistArgs &a, uint32_t n_select, int n_sm, cudaStream_t st);
constexpr int kTracebackWarpsPerBlock = 4;
cudaError_t launch_traceback(const TracebackArgs &a, int n_blocks, cudaStream_t st);
cudaError_t launch_scan_batch(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem, cudaStream_t st);
cudaError_t scan_batch_occupancy(bool query_in_smem, int warps_per_block, size_t smem, int *blocks_per_sm);
int scan_batch_max_warps_by_registers(bool query_in_smem);
cudaError_t gapped_occupancy(int *blocks_per_sm);
// The gapped stage as prep, lane-parallel DP and finishing kernels (batched
// passes of many queries); n_blocks as for launch_gapped, the DP kernel
// fills n_sm SMs. Results equal launch_gapped's.
cudaError_t launch_gapped_split(const GappedArgs &a, int n_blocks, int n_sm, cudaStream_t st);

// Host helpers (host.cpp).
extern const int32_t kBlosum62[kAlphabet][kAlphabet];
// Word lookup of a query: cell_start[kWords + 1], offsets ascending per cell.
int build_lookup(const uint8_t *query, int32_t qlen, int32_t threshold,
                 uint32_t *cell_start, uint16_t **offsets, uint32_t *n_offsets);
// The scan kernel's per-word tables from cell_start: packed cells
// (start << 8 | min(count, 255); 255 sends the kernel to cell_start) and the
// word-presence bitset (kPresenceWords words, overwritten).
void pack_word_cells(const uint32_t *cell_start, uint32_t *pack, uint32_t *presence);
int default_params(int32_t qlen, uint64_t db_len, uint32_t db_n, double evalue,
                   blaze_params *out);

}  // namespace blaze

#define BLAZE_CUDA_TRY(expr)                                  \
    do {                                                      \
        cudaError_t err__ = (expr);                           \
        if (err__ != cudaSuccess) {                           \
            last_cuda_error(err__);                           \
            return err__ == cudaErrorMemoryAllocation         \
                       ? BLAZE_ERR_OUT_OF_MEMORY              \
                       : BLAZE_ERR_CUDA;                      \
        }                                                     \
    } while (0)

void last_cuda_error(cudaError_t e);
