// handles.h -- the library's handle types (database, query, search context,
// query batch) and the device buffers they own, shared by the host-side
// translation units (api.cu, batch.cu, traceback_host.cu, server.cpp via the
// C ABI only).
#pragma once
#include <cstdint>
#include <map>
#include <vector>

#include "blaze_prelim.h"
#include "common.cuh"

using namespace blaze;

constexpr uint32_t kMaxSubjectLength = (1u << 28) - 64;  // diagonal table encoding limit
constexpr int32_t kMaxQueryLength = 32000;                // diagonal table must fit shared memory
constexpr uint32_t kInitialScratchCap = 1024;             // init hits per subject before a rerun

struct blaze_db {
    int device = 0;
    uint8_t *d_res = nullptr;
    uint64_t *d_off = nullptr;
    uint32_t *d_oid = nullptr;     // sorted index -> OID (the hit-list tie rule)
    uint64_t total = 0;
    uint32_t n = 0;
    uint32_t max_len = 0;
    std::vector<uint32_t> oid_of;  // sorted index -> OID
    std::vector<uint32_t> sorted_of;  // OID -> sorted index
    std::vector<uint64_t> h_off;   // offsets of the length-sorted copy (host)
};

struct blaze_query {
    int device = 0;
    int32_t qlen = 0;
    int32_t threshold = 0;
    uint64_t upload_bytes = 0;  // host->device bytes of the tables
    uint8_t *d_q = nullptr;
    uint32_t *d_cell_start = nullptr;
    uint32_t *d_cell_pack = nullptr;
    uint32_t *d_presence = nullptr;
    uint16_t *d_cell_off = nullptr;
    uint32_t n_off = 0;
};

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    int ensure(size_t want) {
        if (want <= n) return BLAZE_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        BLAZE_CUDA_TRY(cudaMalloc(&p, sizeof(T) * std::max<size_t>(want, 1)));
        n = want;
        return BLAZE_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct blaze_search {
    blaze_db *db = nullptr;
    cudaStream_t stream = nullptr;
    int n_sm = 0;
    // per-run capacities
    uint32_t scratch_cap = kInitialScratchCap;
    unsigned long long init_cap = 0, out_cap = 0;
    DevBuf<InitHit> scratch, init_out, sorted;
    DevBuf<WorkItem> work;
    DevBuf<DevHsp> saved, out;
    DevBuf<int32_t> dp;
    DevBuf<InitHit> init_sorted;
    DevBuf<DpTask> dtask;
    DevBuf<int4> dres;
    DevCounters *d_cnt = nullptr;
    DevCounters *h_cnt = nullptr;  // pinned
    DevHsp *h_out = nullptr;       // pinned
    size_t h_out_n = 0;
    int gapped_blocks = 0;
    std::vector<blaze_hsp> results;
    blaze_stats stats{};
    unsigned long long last_init_count = 0, last_work_count = 0;
    bool last_batched = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // launch shape (blaze_search_set_tuning)
    uint32_t stage_bytes = kScanStageBytes;
    uint32_t tile_residues = 0;  // 0: automatic
    // residue-balanced subject ranges of batched tiles, per tile size
    std::map<uint32_t, DevBuf<uint32_t>> tile_bounds;
    std::map<uint32_t, uint32_t> tile_ranges;
    uint32_t max_warps = 0;
    uint32_t launch_mode = 0;
    uint32_t batch_launch = 0;  // blaze_tuning.batch_launch
    // the per-pass launch sequence as a CUDA graph, and the arguments it was
    // captured with
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<unsigned char> graph_key;
    // batched runs
    unsigned long long work_cap = 0;
    DevBuf<BatchQuery> bq;
    DevBuf<const uint8_t *> bqptr;
    DevBuf<int32_t> bqlen, bcut;
    DevBuf<uint32_t> work_query;
    DevBuf<unsigned long long> cursors;  // one work cursor per scan launch of a pass
    // per-query finishing on the device: reap score, max_hsps, published
    // lists per query, and the hit-list selection's segments
    DevBuf<int32_t> bsmin, bmaxh, sel_limit;
    DevBuf<GroupDesc> groups;
    DevBuf<uint32_t> qkept, seg_off, seg_fill, seg_idx, sel_q;
    DevBuf<unsigned long long> seg_keys;
    GroupDesc *h_groups = nullptr;  // pinned
    size_t h_groups_n = 0;
    // query tables of the one-call entry point, reused across calls
    DevBuf<uint8_t> qt_res;
    DevBuf<uint32_t> qt_cs, qt_pack, qt_pres;
    DevBuf<uint16_t> qt_off;
    unsigned char *h_stage = nullptr;  // pinned staging of those tables
    size_t h_stage_n = 0;
    std::vector<blaze_batch_hsp> batch_results;
    // traceback stage
    DevBuf<TbItem> tb_items;
    DevBuf<TbOut> tb_out;
    DevBuf<uint8_t> tb_dirs;
    DevBuf<int32_t> tb_rows, tb_dp;
    DevBuf<unsigned long long> tb_cursor;
    unsigned long long tb_dir_cap = 1ull << 16;  // direction bytes per warp in a first pass
    std::vector<blaze_aligned_hsp> tb_results;
    std::vector<blaze_batch_aligned_hsp> tb_batch_results;
    const blaze_batch *last_batch = nullptr;  // the batch of the last batched run
};

struct blaze_batch {
    int device = 0;
    uint32_t n = 0;
    int32_t threshold = 0;
    std::vector<int32_t> qlen;
    std::vector<uint64_t> res_off, off_off;  // per query: residues, hit lists
    // device tables; a refilled batch keeps them while they are large enough
    DevBuf<uint8_t> res;
    DevBuf<uint32_t> cell_start, cell_pack, presence;
    DevBuf<uint16_t> cell_off;
    uint8_t *d_res = nullptr;
    uint32_t *d_cell_start = nullptr, *d_cell_pack = nullptr, *d_presence = nullptr;
    uint16_t *d_cell_off = nullptr;
    uint64_t upload_bytes = 0, device_bytes = 0;
};

inline bool valid_residues(const uint8_t *r, uint64_t n) {
    uint8_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) bad |= static_cast<uint8_t>(r[i] == 0) | static_cast<uint8_t>(r[i] >= kAlphabet);
    return bad == 0;
}

int check_params(const blaze_params *p);
