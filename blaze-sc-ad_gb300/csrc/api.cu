// api.cu -- C ABI of libblaze103: resident database, query tables, and the
// search driver that runs the two device stages and finishes each subject's
// HSP list (E-values, preliminary E-value reap, OID order) on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "handles.h"
#include "internal.h"

namespace {
thread_local cudaError_t g_last_cuda = cudaSuccess;
}  // namespace

void last_cuda_error(cudaError_t e) { g_last_cuda = e; }
int last_cuda_error_code() { return static_cast<int>(g_last_cuda); }
void set_last_cuda_error_code(int code) { g_last_cuda = static_cast<cudaError_t>(code); }

extern "C" const char *blaze_last_cuda_error(void) { return cudaGetErrorString(g_last_cuda); }

extern "C" int blaze_device_count(int *count) {
    if (!count) return BLAZE_ERR_INVALID_ARG;
    *count = 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return BLAZE_OK;
    }
    *count = n;
    return BLAZE_OK;
}

extern "C" int blaze_db_create(int device, const uint8_t *residues, const uint64_t *offsets,
                               uint32_t n_subjects, blaze_db **out) try {
    if (!out || !offsets || (n_subjects > 0 && !residues)) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    blaze_device_count(&ndev);
    if (ndev == 0) return BLAZE_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return BLAZE_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n_subjects; ++i) {
        if (offsets[i + 1] < offsets[i]) return BLAZE_ERR_INVALID_ARG;
        if (offsets[i + 1] - offsets[i] > kMaxSubjectLength) return BLAZE_ERR_LIMIT;
    }
    const uint64_t base = offsets[0], total = offsets[n_subjects] - base;
    if (!valid_residues(residues + base, total)) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(device));
    auto *db = new blaze_db();
    db->device = device;
    db->n = n_subjects;
    db->total = total;
    // length-sorted order (stable: equal lengths keep OID order)
    std::vector<uint32_t> order(n_subjects);
    std::iota(order.begin(), order.end(), 0u);
    auto len = [&](uint32_t i) { return offsets[i + 1] - offsets[i]; };
    bool sorted = true;
    for (uint32_t i = 1; i < n_subjects && sorted; ++i) sorted = len(i - 1) <= len(i);
    if (!sorted) std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return len(a) < len(b); });
    db->oid_of = order;
    db->sorted_of.resize(n_subjects);
    for (uint32_t k = 0; k < n_subjects; ++k) db->sorted_of[order[k]] = k;
    std::vector<uint64_t> off(n_subjects + 1);
    off[0] = 0;
    for (uint32_t k = 0; k < n_subjects; ++k) {
        off[k + 1] = off[k] + len(order[k]);
        db->max_len = std::max<uint32_t>(db->max_len, static_cast<uint32_t>(len(order[k])));
    }
    int rc = BLAZE_OK;
    do {
        cudaError_t e = cudaMalloc(&db->d_res, total + 64);
        if (e == cudaSuccess) e = cudaMalloc(&db->d_off, sizeof(uint64_t) * (n_subjects + 1));
        if (e == cudaSuccess) e = cudaMalloc(&db->d_oid, sizeof(uint32_t) * std::max<uint32_t>(n_subjects, 1));
        if (e != cudaSuccess) {
            last_cuda_error(e);
            rc = e == cudaErrorMemoryAllocation ? BLAZE_ERR_OUT_OF_MEMORY : BLAZE_ERR_CUDA;
            break;
        }
        if (sorted) {
            e = cudaMemcpy(db->d_res, residues + base, total, cudaMemcpyHostToDevice);
        } else {
            std::vector<uint8_t> tmp(total);
            for (uint32_t k = 0; k < n_subjects; ++k)
                std::memcpy(tmp.data() + off[k], residues + offsets[order[k]], len(order[k]));
            e = cudaMemcpy(db->d_res, tmp.data(), total, cudaMemcpyHostToDevice);
        }
        if (e == cudaSuccess) e = cudaMemset(db->d_res + total, 0, 64);
        if (e == cudaSuccess) e = cudaMemcpy(db->d_off, off.data(), sizeof(uint64_t) * (n_subjects + 1), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n_subjects)
            e = cudaMemcpy(db->d_oid, order.data(), sizeof(uint32_t) * n_subjects, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            last_cuda_error(e);
            rc = BLAZE_ERR_CUDA;
        }
    } while (false);
    if (rc != BLAZE_OK) {
        blaze_db_free(db);
        return rc;
    }
    db->h_off.swap(off);
    *out = db;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_db_free(blaze_db *db) {
    if (!db) return BLAZE_OK;
    cudaSetDevice(db->device);
    if (db->d_res) cudaFree(db->d_res);
    if (db->d_off) cudaFree(db->d_off);
    if (db->d_oid) cudaFree(db->d_oid);
    delete db;
    return BLAZE_OK;
}

extern "C" int blaze_db_info(const blaze_db *db, uint64_t *total, uint32_t *n, uint32_t *max_len) {
    if (!db) return BLAZE_ERR_INVALID_ARG;
    if (total) *total = db->total;
    if (n) *n = db->n;
    if (max_len) *max_len = db->max_len;
    return BLAZE_OK;
}

// A query's word tables on the host: cell_start (kWords + 1 prefix offsets),
// the packed cells (start << 8 | min(count, 255); 255: look at cell_start),
// the word-presence bitset and the hit lists (query offsets).
struct QueryTables {
    std::vector<uint32_t> cs, pack, pres;
    uint16_t *offs = nullptr;  // malloc'd by build_lookup
    uint32_t n_off = 0;
    ~QueryTables() { std::free(offs); }
};

static int query_tables(const uint8_t *query, int32_t length, int32_t word_threshold, QueryTables &t) {
    t.cs.assign(kWords + 1, 0u);
    int rc = build_lookup(query, length, word_threshold, t.cs.data(), &t.offs, &t.n_off);
    if (rc != BLAZE_OK) return rc;
    t.pack.resize(kWords);
    t.pres.resize(kPresenceWords);
    pack_word_cells(t.cs.data(), t.pack.data(), t.pres.data());
    return BLAZE_OK;
}

static uint64_t query_upload_bytes(int32_t length, uint32_t n_off) {
    return static_cast<uint64_t>(length) + sizeof(uint32_t) * (2 * kWords + 1 + kPresenceWords) +
           sizeof(uint16_t) * n_off;
}

extern "C" int blaze_query_create(const blaze_db *db, const uint8_t *query, int32_t length,
                                  int32_t word_threshold, blaze_query **out) try {
    if (!db || !query || !out || length <= 0) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    if (length > kMaxQueryLength) return BLAZE_ERR_LIMIT;
    if (!valid_residues(query, static_cast<uint64_t>(length))) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(db->device));
    QueryTables t;
    int rc = query_tables(query, length, word_threshold, t);
    if (rc != BLAZE_OK) return rc;
    auto *q = new blaze_query();
    q->device = db->device;
    q->qlen = length;
    q->threshold = word_threshold;
    q->n_off = t.n_off;
    cudaError_t e = cudaMalloc(&q->d_q, static_cast<size_t>(length) + 64);
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_start, sizeof(uint32_t) * (kWords + 1));
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_off, sizeof(uint16_t) * std::max<uint32_t>(t.n_off, 1));
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_pack, sizeof(uint32_t) * kWords);
    if (e == cudaSuccess) e = cudaMalloc(&q->d_presence, sizeof(uint32_t) * kPresenceWords);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_cell_pack, t.pack.data(), sizeof(uint32_t) * kWords, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_presence, t.pres.data(), sizeof(uint32_t) * kPresenceWords, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_q, query, length, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(q->d_q + length, 0, 64);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_cell_start, t.cs.data(), sizeof(uint32_t) * (kWords + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && t.n_off) e = cudaMemcpy(q->d_cell_off, t.offs, sizeof(uint16_t) * t.n_off, cudaMemcpyHostToDevice);
    q->upload_bytes = query_upload_bytes(length, t.n_off);
    if (e != cudaSuccess) {
        last_cuda_error(e);
        blaze_query_free(q);
        return e == cudaErrorMemoryAllocation ? BLAZE_ERR_OUT_OF_MEMORY : BLAZE_ERR_CUDA;
    }
    *out = q;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_query_free(blaze_query *q) {
    if (!q) return BLAZE_OK;
    cudaSetDevice(q->device);
    if (q->d_q) cudaFree(q->d_q);
    if (q->d_cell_start) cudaFree(q->d_cell_start);
    if (q->d_cell_pack) cudaFree(q->d_cell_pack);
    if (q->d_presence) cudaFree(q->d_presence);
    if (q->d_cell_off) cudaFree(q->d_cell_off);
    delete q;
    return BLAZE_OK;
}

extern "C" int blaze_search_create(blaze_db *db, blaze_search **out) try {
    if (!db || !out) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    BLAZE_CUDA_TRY(cudaSetDevice(db->device));
    auto *s = new blaze_search();
    s->db = db;
    cudaError_t e = cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, db->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_cnt, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_cnt, sizeof(DevCounters));
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&s->ev[i]);
    int per_sm = 0;
    if (e == cudaSuccess) e = gapped_occupancy(&per_sm);
    if (e != cudaSuccess) {
        last_cuda_error(e);
        blaze_search_free(s);
        return BLAZE_ERR_CUDA;
    }
    s->gapped_blocks = s->n_sm * std::min(std::max(per_sm, 1), 8);
    s->init_cap = std::max<unsigned long long>(1ull << 20, db->n / 8);
    s->work_cap = std::max<unsigned long long>(1ull << 20, db->n / 4);
    s->out_cap = std::max<unsigned long long>(1ull << 20, db->n / 16);
    // Starting capacities can be lowered (e.g. to exercise the grow-and-repeat
    // path); they grow on demand either way.
    if (const char *v = std::getenv("BLAZE_INITIAL_SCRATCH_CAP")) s->scratch_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_INIT_CAP")) s->init_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_OUT_CAP")) s->out_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_WORK_CAP")) s->work_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_TRACEBACK_CAP")) s->tb_dir_cap = std::max(64, std::atoi(v));
    *out = s;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_free(blaze_search *s) {
    if (!s) return BLAZE_OK;
    cudaSetDevice(s->db->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    for (auto &kv : s->tile_bounds) kv.second.release();
    s->scratch.release();
    s->init_out.release();
    s->init_sorted.release();
    s->dtask.release();
    s->dres.release();
    s->sorted.release();
    s->work.release();
    s->saved.release();
    s->out.release();
    s->dp.release();
    s->bq.release();
    s->bqptr.release();
    s->bqlen.release();
    s->bcut.release();
    s->work_query.release();
    s->cursors.release();
    s->bsmin.release();
    s->bmaxh.release();
    s->sel_limit.release();
    s->groups.release();
    s->qkept.release();
    s->seg_off.release();
    s->seg_fill.release();
    s->seg_idx.release();
    s->sel_q.release();
    s->seg_keys.release();
    s->qt_res.release();
    s->qt_cs.release();
    s->qt_pack.release();
    s->qt_pres.release();
    s->qt_off.release();
    if (s->h_stage) cudaFreeHost(s->h_stage);
    s->tb_items.release();
    s->tb_out.release();
    s->tb_dirs.release();
    s->tb_rows.release();
    s->tb_dp.release();
    s->tb_cursor.release();
    if (s->h_groups) cudaFreeHost(s->h_groups);
    if (s->d_cnt) cudaFree(s->d_cnt);
    if (s->h_cnt) cudaFreeHost(s->h_cnt);
    if (s->h_out) cudaFreeHost(s->h_out);
    for (cudaEvent_t ev : s->ev)
        if (ev) cudaEventDestroy(ev);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return BLAZE_OK;
}

int check_params(const blaze_params *p) {
    if (!p) return BLAZE_ERR_INVALID_ARG;
    if (p->window <= 0 || p->window > (1 << 20) || p->ungapped_xdrop <= 0 || p->gap_open < 0 ||
        p->gap_extend <= 0 || p->gapped_xdrop <= 0 || p->gapped_cutoff <= 0 || p->ungapped_cutoff <= 0)
        return BLAZE_ERR_INVALID_ARG;
    // E-value statistics: E must fall with the score (the reap is a score threshold)
    if (!(p->lambda > 0.0) || !std::isfinite(p->lambda) || !(p->K > 0.0) || !std::isfinite(p->K) ||
        !(p->eff_searchsp >= 0.0) || !std::isfinite(p->eff_searchsp) || std::isnan(p->prelim_evalue))
        return BLAZE_ERR_INVALID_ARG;
    return BLAZE_OK;
}

// The preliminary reap drops an HSP when eff_searchsp * K * exp(-lambda * S)
// exceeds prelim_evalue. E falls with S, so on the scores a gapped HSP can
// have (1 and up) it keeps exactly those from the smallest passing S, found
// by bisection over the same expression.
static int32_t reap_min_score(const blaze_params &p) {
    auto keeps = [&p](int64_t S) {
        return !(p.eff_searchsp * p.K * std::exp(-p.lambda * static_cast<double>(S)) > p.prelim_evalue);
    };
    int64_t lo = 1, hi = INT32_MAX;  // keeps(hi) or no score passes
    if (keeps(lo)) return 1;
    if (!keeps(hi)) return INT32_MAX;
    while (hi - lo > 1) {  // !keeps(lo), keeps(hi)
        const int64_t mid = lo + (hi - lo) / 2;
        (keeps(mid) ? hi : lo) = mid;
    }
    return static_cast<int32_t>(hi);
}

// What one run searches: one query, or a batch with one parameter set per
// query.
struct RunSpec {
    const blaze_query *q = nullptr;
    const blaze_batch *b = nullptr;
    const blaze_params *p = nullptr;
    std::vector<int32_t> smin;  // per query: the reap's lowest kept score
    std::vector<uint32_t> border;  // batched: query indices in launch (length) order
};

// One pass of both stages; fills s->h_cnt.
// One pass's launch sequence: counter reset, scan kernel, gapped kernel and
// the counter read-back, with the timing events between them.
struct ScanLaunch {
    ScanArgs sa;
    int blocks, warps_per_block;
    size_t smem_bytes;
    bool tiles;  // the batched (tiled) kernel, else the single-query one
};

struct PassLaunch {
    std::vector<ScanLaunch> scans;
    const GappedArgs *ga;
    bool batched;
    bool split;  // the gapped stage as prep, lane-parallel DP and finishing kernels
};

// Batched passes of at least this many queries run the gapped stage with one
// lane per DP: they hold enough DPs (thousands per SM) for its throughput,
// while a pass of one or a few queries finishes sooner with a warp per
// subject (a lane's DP takes too long for a pass that gives each lane one or
// two of them).
constexpr uint32_t kGappedSplitMinQueries = 16;

static cudaError_t enqueue_pass(blaze_search *s, const PassLaunch &pl, unsigned event_flags) {
    cudaError_t e = cudaMemsetAsync(s->d_cnt, 0, sizeof(DevCounters), s->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s->cursors.p, 0, sizeof(unsigned long long) * pl.scans.size(), s->stream);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(s->ev[1], s->stream, event_flags);
    for (const ScanLaunch &l : pl.scans) {
        if (e != cudaSuccess) break;
        e = l.tiles ? launch_scan_batch(l.sa, l.blocks, l.warps_per_block, l.smem_bytes, s->stream)
                       : launch_scan(l.sa, l.blocks, l.warps_per_block, l.smem_bytes, s->stream);
    }
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(s->ev[2], s->stream, event_flags);
    if (e == cudaSuccess)
        e = pl.split ? launch_gapped_split(*pl.ga, s->gapped_blocks, s->n_sm, s->stream)
                     : launch_gapped(*pl.ga, s->gapped_blocks, s->stream);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(s->ev[3], s->stream, event_flags);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->h_cnt, s->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, s->stream);
    return e;
}

static int launch_pass_direct(blaze_search *s, const PassLaunch &pl) {
    BLAZE_CUDA_TRY(enqueue_pass(s, pl, cudaEventRecordDefault));
    return BLAZE_OK;
}

// Replays the pass from a CUDA graph. The graph's kernel arguments are the
// ScanArgs/GappedArgs values themselves (every buffer they point to keeps its
// address while it is not regrown), so a pass whose arguments and launch
// shapes equal those of the captured one replays it; otherwise the sequence
// is captured again and the executable graph updated in place (or rebuilt
// when the update is refused). Capture is thread-local, so other host
// threads may allocate meanwhile.
static int launch_pass_graph(blaze_search *s, const PassLaunch &pl) {
    std::vector<unsigned char> key;
    auto put = [&key](const void *p, size_t n) {
        const auto *c = static_cast<const unsigned char *>(p);
        key.insert(key.end(), c, c + n);
    };
    const int64_t head[3] = {pl.batched, pl.split, s->gapped_blocks};
    put(head, sizeof(head));
    for (const ScanLaunch &l : pl.scans) {
        put(&l.sa, sizeof(ScanArgs));
        const int64_t shape[3] = {l.blocks, l.warps_per_block, static_cast<int64_t>(l.smem_bytes)};
        put(shape, sizeof(shape));
    }
    put(pl.ga, sizeof(GappedArgs));
    if (s->graph_exec && key == s->graph_key) {
        BLAZE_CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
        s->stats.graph_replays++;
        return BLAZE_OK;
    }
    BLAZE_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = enqueue_pass(s, pl, cudaEventRecordExternal);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        s->graph_key.clear();
        BLAZE_CUDA_TRY(e != cudaSuccess ? e : ec);
    }
    bool updated = false;
    if (s->graph_exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(s->graph_exec, g, &info) == cudaSuccess) {
            updated = true;
        } else {
            cudaGetLastError();  // a refused update is not an error: rebuild
            cudaGraphExecDestroy(s->graph_exec);
            s->graph_exec = nullptr;
        }
    }
    cudaError_t ei = cudaSuccess;
    if (!updated) ei = cudaGraphInstantiate(&s->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        s->graph_exec = nullptr;
        s->graph_key.clear();
        BLAZE_CUDA_TRY(ei);
    }
    s->graph_key.swap(key);
    s->stats.graph_builds++;
    BLAZE_CUDA_TRY(cudaGraphLaunch(s->graph_exec, s->stream));
    return BLAZE_OK;
}

// One scan launch of a pass: the single-query kernel (a single-query run, or
// one query of a batch), or the batched kernel over a group of a batch's
// queries (queries [first, first + n) of the length-ordered descriptors),
// each with its own shared-memory layout.
struct ScanPlan {
    ScanLayout lay;
    int blocks = 0;
    uint32_t first = 0, n = 1;
    uint32_t tile_residues = 0;
    bool tiles = false;  // batched: tiles of the plan's queries; else one query's launch
};

// Subject ranges of about `target` residues, from the longest subjects down
// (bounds descending, n_ranges + 1 of them), uploaded once per tile size.
static int tile_bounds_for(blaze_search *s, uint32_t target, const uint32_t **bounds, uint32_t *n_ranges) {
    auto it = s->tile_bounds.find(target);
    if (it == s->tile_bounds.end()) {
        const std::vector<uint64_t> &off = s->db->h_off;
        const uint32_t n = s->db->n;
        std::vector<uint32_t> b{n};
        for (uint32_t hi = n; hi > 0;) {
            const uint64_t want = off[hi] > target ? off[hi] - target : 0;
            uint32_t lo = static_cast<uint32_t>(std::lower_bound(off.begin(), off.begin() + hi, want) - off.begin());
            if (lo >= hi) lo = hi - 1;
            b.push_back(lo);
            hi = lo;
        }
        DevBuf<uint32_t> d;
        int rc = d.ensure(b.size());
        if (rc != BLAZE_OK) return rc;
        cudaError_t e = cudaMemcpy(d.p, b.data(), sizeof(uint32_t) * b.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            d.release();
            BLAZE_CUDA_TRY(e);
        }
        s->stats.h2d_bytes += sizeof(uint32_t) * b.size();
        it = s->tile_bounds.emplace(target, d).first;
        s->tile_ranges[target] = static_cast<uint32_t>(b.size() - 1);
    }
    *bounds = it->second.p;
    *n_ranges = s->tile_ranges[target];
    return BLAZE_OK;
}

// One pass of both stages; fills s->h_cnt.
static int run_pass(blaze_search *s, const RunSpec &r, const std::vector<ScanPlan> &plans) {
    blaze_db *db = s->db;
    const blaze_params *p = r.p;
    const bool batched = r.b != nullptr;
    size_t scan_warps = 0;
    for (const ScanPlan &pl : plans)
        scan_warps = std::max(scan_warps, static_cast<size_t>(pl.blocks) * pl.lay.warps_per_block);
    const size_t gapped_warps = static_cast<size_t>(s->gapped_blocks) * kGappedWarpsPerBlock;
    const size_t work_cap = batched ? s->work_cap : std::max<uint32_t>(db->n, 1);
    int rc;
    if ((rc = s->scratch.ensure(scan_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->sorted.ensure(gapped_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->saved.ensure(gapped_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->init_out.ensure(s->init_cap)) != BLAZE_OK) return rc;
    if ((rc = s->work.ensure(work_cap)) != BLAZE_OK) return rc;
    if ((rc = s->out.ensure(s->out_cap)) != BLAZE_OK) return rc;
    const uint32_t nq = batched ? r.b->n : 1u;
    const bool split = batched && nq >= kGappedSplitMinQueries;
    if (split) {  // per init-hit slot: ordered init hit, DP task, two DP results
        if ((rc = s->init_sorted.ensure(s->init_cap)) != BLAZE_OK) return rc;
        if ((rc = s->dtask.ensure(s->init_cap)) != BLAZE_OK) return rc;
        if ((rc = s->dres.ensure(2 * s->init_cap)) != BLAZE_OK) return rc;
    }
    if ((rc = s->groups.ensure(s->out_cap)) != BLAZE_OK) return rc;  // a published list holds >= 1 HSP
    if ((rc = s->qkept.ensure(nq)) != BLAZE_OK) return rc;
    if (batched && (rc = s->work_query.ensure(work_cap)) != BLAZE_OK) return rc;
    // DP rows of the longest subject plus 2, even so that each warp's H and E
    // rows start 8-byte aligned (the DP reads and writes column pairs)
    const size_t dp_stride = (static_cast<size_t>(std::max<uint32_t>(db->max_len, 1)) + 3) & ~size_t{1};
    if ((rc = s->dp.ensure(gapped_warps * 2 * dp_stride)) != BLAZE_OK) return rc;
    if ((rc = s->cursors.ensure(plans.size())) != BLAZE_OK) return rc;

    PassLaunch pl;
    pl.batched = batched;
    pl.split = split;
    for (const ScanPlan &plan : plans) {
        const ScanLayout &lay = plan.lay;
        ScanLaunch l;
        ScanArgs &sa = l.sa;
        std::memset(&sa, 0, sizeof(sa));  // whole bytes: the graph key compares them
        l.blocks = plan.blocks;
        l.warps_per_block = lay.warps_per_block;
        l.smem_bytes = lay.smem_bytes;
        sa.res = db->d_res;
        sa.off = db->d_off;
        sa.n_subj = db->n;
        sa.window = p->window;
        sa.xdrop = p->ungapped_xdrop;
        sa.diag_entries = lay.diag_entries;
        sa.diag_magic = lay.diag_magic;
        sa.diag_bytes = lay.diag_bytes;
        sa.diag_entries_max = lay.diag_entries;
        sa.stage_bytes = lay.stage_bytes;
        sa.query_smem_bytes = lay.query_smem_bytes;
        sa.warp_smem_bytes = lay.warp_smem_bytes;
        sa.smem_bytes = static_cast<uint32_t>(lay.smem_bytes);
        sa.scratch = s->scratch.p;
        sa.scratch_cap = s->scratch_cap;
        sa.init_out = s->init_out.p;
        sa.init_cap = s->init_cap;
        sa.work = s->work.p;
        sa.work_cap = work_cap;
        sa.cnt = s->d_cnt;
        sa.cursor = s->cursors.p + pl.scans.size();
        l.tiles = plan.tiles;
        if (batched && !plan.tiles) {
            // one query of the batch with the single-query kernel; its work
            // items carry the query's batch index
            const uint32_t i = r.border[plan.first];
            const blaze_batch *b = r.b;
            sa.q = b->d_res + b->res_off[i];
            sa.qlen = b->qlen[i];
            sa.cell_start = b->d_cell_start + static_cast<size_t>(i) * (kWords + 1);
            sa.cell_pack = b->d_cell_pack + static_cast<size_t>(i) * kWords;
            sa.presence = b->d_presence + static_cast<size_t>(i) * kPresenceWords;
            sa.cell_off = b->d_cell_off + b->off_off[i];
            sa.cutoff = r.p[i].ungapped_cutoff;
            sa.n_queries = 1;
            sa.query_index = i;
            sa.work_query = s->work_query.p;
        } else if (batched) {
            sa.queries = s->bq.p + plan.first;
            sa.n_queries = plan.n;
            // a tile is one block's work: tile_residues per warp
            const uint32_t block_tile = static_cast<uint32_t>(std::min<uint64_t>(
                static_cast<uint64_t>(plan.tile_residues) * static_cast<uint64_t>(lay.warps_per_block), 1u << 31));
            if ((rc = tile_bounds_for(s, block_tile, &sa.tile_bounds, &sa.n_ranges)) != BLAZE_OK) return rc;
            sa.work_query = s->work_query.p;
        } else {
            const blaze_query *q = r.q;
            sa.q = q->d_q;
            sa.qlen = q->qlen;
            sa.cell_start = q->d_cell_start;
            sa.cell_pack = q->d_cell_pack;
            sa.presence = q->d_presence;
            sa.cell_off = q->d_cell_off;
            sa.cutoff = p->ungapped_cutoff;
            sa.n_queries = 1;
        }
        pl.scans.push_back(l);
    }

    GappedArgs ga;
    std::memset(&ga, 0, sizeof(ga));
    ga.res = db->d_res;
    ga.off = db->d_off;
    ga.init_in = s->init_out.p;
    ga.work = s->work.p;
    ga.work_cap = work_cap;
    ga.init_cap = s->init_cap;
    ga.n_subj = db->n;
    ga.n_queries = nq;
    ga.sorted = s->sorted.p;
    ga.saved = s->saved.p;
    ga.cap = s->scratch_cap;
    ga.dp = s->dp.p;
    ga.dp_stride = static_cast<uint32_t>(dp_stride);
    ga.gap_open = p->gap_open;
    ga.gap_extend = p->gap_extend;
    ga.xdrop = p->gapped_xdrop;
    ga.out = s->out.p;
    ga.out_cap = s->out_cap;
    ga.oid = db->d_oid;
    ga.groups = s->groups.p;
    ga.qkept = s->qkept.p;
    ga.cnt = s->d_cnt;
    if (split) {
        ga.init_sorted = s->init_sorted.p;
        ga.dtask = s->dtask.p;
        ga.dres = s->dres.p;
    }
    if (batched) {
        ga.work_query = s->work_query.p;
        ga.batch_q = s->bqptr.p;
        ga.batch_qlen = s->bqlen.p;
        ga.batch_cutoff = s->bcut.p;
        ga.batch_smin = s->bsmin.p;
        ga.batch_max_hsps = s->bmaxh.p;
    } else {
        ga.q = r.q->d_q;
        ga.qlen = r.q->qlen;
        ga.cutoff = p->gapped_cutoff;
        ga.smin = r.smin[0];
        ga.max_hsps = p->max_hsps;
    }
    pl.ga = &ga;
    BLAZE_CUDA_TRY(cudaMemsetAsync(s->qkept.p, 0, sizeof(uint32_t) * nq, s->stream));
    const bool graph = s->launch_mode == 2 || (s->launch_mode == 0 && batched);
    if ((rc = graph ? launch_pass_graph(s, pl) : launch_pass_direct(s, pl)) != BLAZE_OK) return rc;
    s->stats.kernel_launches += static_cast<uint32_t>(pl.scans.size()) + 1;
    s->stats.d2h_bytes += sizeof(DevCounters);
    BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return BLAZE_OK;
}

template <typename T>
static int ensure_pinned(T *&p, size_t &n, size_t want) {
    if (want <= n) return BLAZE_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    BLAZE_CUDA_TRY(cudaMallocHost(&p, sizeof(T) * want));
    n = want;
    return BLAZE_OK;
}

// Runs both stages (growing buffers and repeating a pass that overflowed),
// copies the HSPs back and finishes them: E-values, preliminary reap, order
// by (query, OID).
static int run_search(blaze_search *s, const RunSpec &spec, uint64_t *n_hsps) {
    blaze_db *db = s->db;
    const blaze_params *p0 = spec.p;
    const bool batched = spec.b != nullptr;
    const uint32_t nq = batched ? spec.b->n : 1;
    RunSpec r = spec;
    r.smin.resize(nq);
    for (uint32_t i = 0; i < nq; ++i) r.smin[i] = reap_min_score(r.p[i]);
    s->results.clear();
    s->batch_results.clear();
    s->stats = blaze_stats{};
    if (n_hsps) *n_hsps = 0;

    constexpr size_t kSmemBudget = 220 * 1024;
    const int reg_cap = batched ? std::min(scan_batch_max_warps_by_registers(true),
                                           scan_batch_max_warps_by_registers(false))
                                : scan_max_warps_by_registers(r.q->qlen <= static_cast<int32_t>(kQuerySmemMax));
    const int warp_cap = s->max_warps ? std::min(reg_cap, static_cast<int>(s->max_warps)) : reg_cap;
    // layout of one single-query scan launch
    auto layout_for = [&](int32_t max_qlen) {
        return scan_layout(max_qlen, p0->window, s->stage_bytes, kSmemBudget, warp_cap);
    };
    // layout of one batched scan launch over queries of up to `longest`
    // residues: shared memory for all the block's warps at the longest query
    // when that fits the budget, else the whole budget (at least one warp);
    // each tile runs as many warps as fit for its own query
    auto batch_layout_for = [&](int32_t longest) {
        ScanLayout l{};
        const uint32_t stage_region = (s->stage_bytes + 32u + 15u) & ~15u;
        auto warp_bytes = [&](int32_t qlen) {
            const uint32_t e = static_cast<uint32_t>(qlen + p0->window + 3) & ~3u;
            return static_cast<size_t>(((4u * e + 15u) & ~15u) + 2u * kDeferCap * sizeof(uint2) +
                                       kSeedCap * sizeof(int4) + stage_region);
        };
        const int w = std::max(1, std::min(warp_cap, kScanMaxWarpsPerBlock));
        l.query_smem_bytes = longest <= kQuerySmemMax ? (static_cast<uint32_t>(longest) + 15u) & ~15u : 0u;
        const size_t regions = kScanMatBytes + kScanPresenceBytes + l.query_smem_bytes + 16u * static_cast<size_t>(w);
        l.smem_bytes = std::max(std::min(kSmemBudget, regions + static_cast<size_t>(w) * warp_bytes(longest)),
                                regions + warp_bytes(longest));
        l.warps_per_block = w;
        l.stage_bytes = s->stage_bytes;
        l.diag_entries = static_cast<uint32_t>(longest + p0->window + 3) & ~3u;
        l.diag_magic = static_cast<uint32_t>((1ull << 32) / l.diag_entries + 1);
        l.diag_bytes = 4u * l.diag_entries;
        l.warp_smem_bytes = static_cast<uint32_t>(warp_bytes(longest));
        return l;
    };
    // Batched: one scan launch for the queries whose residues fit the
    // block's shared-memory copy and one for any longer ones (their tiles
    // size the warps' tables per query).
    std::vector<uint32_t> order(nq);
    std::iota(order.begin(), order.end(), 0u);
    if (batched)
        std::stable_sort(order.begin(), order.end(),
                         [&](uint32_t a, uint32_t b) { return r.b->qlen[a] < r.b->qlen[b]; });
    auto qlen_at = [&](uint32_t k) { return batched ? r.b->qlen[order[k]] : r.q->qlen; };
    std::vector<ScanPlan> plans;
    // A launch's shared memory fixes the SM's L1 share for all of it, and the
    // L1 keeps the word tables the finder reads per position; so batched
    // queries are grouped by the shared-memory step (of the SM's carve-out
    // choices) that all the block's warps need for them, each group one launch
    // sized for its longest query -- what a single-query launch does per query.
    auto smem_step = [&](int32_t qlen) {
        constexpr size_t kSteps[] = {100u << 10, 132u << 10, 164u << 10, 196u << 10};
        const size_t need = batch_layout_for(qlen).smem_bytes;
        int k = 0;
        while (k < 4 && need > kSteps[k]) ++k;
        return k + (qlen > kQuerySmemMax ? 8 : 0);  // longer queries stay in global memory: own launch
    };
    // batched runs of few queries, or on a large database, launch the
    // single-query kernel once per query (a query alone fills the GPU there,
    // and that kernel is the faster per residue); the tiles pay off where
    // many per-query launches would each be short
    constexpr uint64_t kPerQueryLaunchResidues = 1ull << 27;
    constexpr uint32_t kPerQueryLaunchQueries = 16;
    const bool per_query = batched && (s->batch_launch == 2 ||
                                       (s->batch_launch == 0 && (db->total >= kPerQueryLaunchResidues ||
                                                                 nq <= kPerQueryLaunchQueries)));
    r.border = order;
    for (uint32_t i = 0; i < nq;) {
        uint32_t j = i + 1;
        if (batched && !per_query) {
            const int step = smem_step(qlen_at(i));
            while (j < nq && smem_step(qlen_at(j)) == step) ++j;
        }
        ScanPlan pl;
        pl.tiles = batched && !per_query;
        pl.lay = pl.tiles ? batch_layout_for(qlen_at(j - 1)) : layout_for(qlen_at(j - 1));
        pl.first = i;
        pl.n = j - i;
        if (pl.lay.smem_bytes > 227 * 1024 - 64) return BLAZE_ERR_LIMIT;  // the opt-in limit less static shared memory
        int per_sm = 0;
        if (pl.tiles) {
            BLAZE_CUDA_TRY(scan_batch_occupancy(pl.lay.query_smem_bytes != 0, pl.lay.warps_per_block, pl.lay.smem_bytes,
                                                &per_sm));
        } else {
            BLAZE_CUDA_TRY(scan_occupancy(pl.lay.query_smem_bytes != 0, pl.lay.warps_per_block, pl.lay.smem_bytes, &per_sm));
        }
        if (per_sm < 1) return BLAZE_ERR_LIMIT;
        pl.blocks = s->n_sm * per_sm;
        if (pl.tiles) {
            if (s->tile_residues) {
                pl.tile_residues = s->tile_residues;
            } else {
                // about 16 tiles per block (its warps wait for the last one
                // at each tile's end, so larger tiles waste less), at most
                // kMaxTileResidues per warp; a power of two so that few
                // distinct bound tables exist
                const uint64_t per_block = db->total * pl.n / (16ull * static_cast<uint64_t>(pl.blocks));
                uint64_t t = std::max<uint64_t>(per_block / static_cast<uint64_t>(pl.lay.warps_per_block), 1);
                t = std::min<uint64_t>(t, kMaxTileResidues);
                uint32_t pow2 = 1;
                while (static_cast<uint64_t>(pow2) * 2 <= t) pow2 *= 2;
                pl.tile_residues = pow2;
            }
        }
        plans.push_back(pl);
        i = j;
    }

    if (batched) {
        // per-query descriptors of this run in length order (cutoffs come from
        // the parameters); the per-query arrays of the gapped stage stay in
        // batch order
        std::vector<BatchQuery> bq(nq);
        std::vector<const uint8_t *> qp(nq);
        std::vector<int32_t> ql(nq), cut(nq), mh(nq);
        for (uint32_t k = 0; k < nq; ++k) {
            const uint32_t i = order[k];
            const blaze_params &pi = r.p[i];
            BatchQuery &d = bq[k];
            d.q = r.b->d_res + r.b->res_off[i];
            d.qlen = r.b->qlen[i];
            d.ungapped_cutoff = pi.ungapped_cutoff;
            d.cell_start = r.b->d_cell_start + static_cast<size_t>(i) * (kWords + 1);
            d.cell_pack = r.b->d_cell_pack + static_cast<size_t>(i) * kWords;
            d.presence = r.b->d_presence + static_cast<size_t>(i) * kPresenceWords;
            d.cell_off = r.b->d_cell_off + r.b->off_off[i];
            d.diag_entries = static_cast<uint32_t>(d.qlen + pi.window + 3) & ~3u;
            d.diag_magic = static_cast<uint32_t>((1ull << 32) / d.diag_entries + 1);
            d.index = i;
            qp[i] = d.q;
            ql[i] = d.qlen;
            cut[i] = pi.gapped_cutoff;
            mh[i] = pi.max_hsps;
        }
        int rc;
        if ((rc = s->bq.ensure(nq)) != BLAZE_OK) return rc;
        if ((rc = s->bqptr.ensure(nq)) != BLAZE_OK) return rc;
        if ((rc = s->bqlen.ensure(nq)) != BLAZE_OK) return rc;
        if ((rc = s->bcut.ensure(nq)) != BLAZE_OK) return rc;
        if ((rc = s->bsmin.ensure(nq)) != BLAZE_OK) return rc;
        if ((rc = s->bmaxh.ensure(nq)) != BLAZE_OK) return rc;
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bq.p, bq.data(), sizeof(BatchQuery) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bqptr.p, qp.data(), sizeof(const uint8_t *) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bqlen.p, ql.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bcut.p, cut.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bsmin.p, r.smin.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->bmaxh.p, mh.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s->stream));
        BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
        s->stats.h2d_bytes += (sizeof(BatchQuery) + sizeof(const uint8_t *) + 4 * sizeof(int32_t)) * nq;
    }

    DevCounters c{};
    int rc;
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[0], s->stream));
    for (int attempt = 0;; ++attempt) {
        if ((rc = run_pass(s, r, plans)) != BLAZE_OK) return rc;
        c = *s->h_cnt;
        {
            float ms = 0.f;
            BLAZE_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[2], s->ev[3]));
            s->stats.gapped_ms = ms;
        }
        // the DP rows fit the longest subject and the scan's init hits lie in
        // their sequences, so these two are consistency failures here
        if (c.flags & (kFlagBadState | kFlagSubjectTooLong | kFlagBadInitHit)) return BLAZE_ERR_INTERNAL;
        bool again = false;
        if (c.overflow_subjects > 0) {
            s->scratch_cap = std::max<uint32_t>(s->scratch_cap * 2, c.max_init_needed + 64);
            again = true;
        }
        if (c.flags & kFlagInitArrayFull) {
            s->init_cap = std::max<unsigned long long>(s->init_cap * 2, c.init_count + c.init_count / 4 + 1024);
            again = true;
        }
        if (c.flags & kFlagOutArrayFull) {
            s->out_cap = std::max<unsigned long long>(s->out_cap * 2, c.out_count + c.out_count / 4 + 1024);
            again = true;
        }
        if (c.flags & kFlagWorkArrayFull) {
            if (!batched) return BLAZE_ERR_INTERNAL;  // one item per subject at most
            s->work_cap = std::max<unsigned long long>(s->work_cap * 2, c.work_count + c.work_count / 4 + 1024);
            again = true;
        }
        if (!again) break;
        if (attempt >= 8) return BLAZE_ERR_INTERNAL;
        s->stats.reruns++;
    }

    // hit lists: a query keeping more subjects than its hitlist_size keeps
    // the hitlist_size best on the device (the others' lists get n = 0)
    const size_t n_groups = static_cast<size_t>(c.group_count);
    bool limited = false;
    for (uint32_t i = 0; i < nq; ++i) limited |= r.p[i].hitlist_size > 0;
    if (limited && n_groups) {
        std::vector<uint32_t> kept_per_query(nq);
        BLAZE_CUDA_TRY(cudaMemcpyAsync(kept_per_query.data(), s->qkept.p, sizeof(uint32_t) * nq,
                                       cudaMemcpyDeviceToHost, s->stream));
        BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
        s->stats.d2h_bytes += sizeof(uint32_t) * nq;
        std::vector<uint32_t> seg(nq + 1, 0), sel;
        std::vector<int32_t> limit(nq);
        for (uint32_t i = 0; i < nq; ++i) {
            limit[i] = r.p[i].hitlist_size;
            const bool selects = limit[i] > 0 && kept_per_query[i] > static_cast<uint32_t>(limit[i]);
            seg[i + 1] = seg[i] + (selects ? kept_per_query[i] : 0u);
            if (selects) sel.push_back(i);
        }
        if (!sel.empty()) {
            int rc2;
            if ((rc2 = s->seg_off.ensure(nq + 1)) != BLAZE_OK) return rc2;
            if ((rc2 = s->seg_fill.ensure(nq)) != BLAZE_OK) return rc2;
            if ((rc2 = s->sel_limit.ensure(nq)) != BLAZE_OK) return rc2;
            if ((rc2 = s->sel_q.ensure(sel.size())) != BLAZE_OK) return rc2;
            if ((rc2 = s->seg_keys.ensure(seg[nq])) != BLAZE_OK) return rc2;
            if ((rc2 = s->seg_idx.ensure(seg[nq])) != BLAZE_OK) return rc2;
            BLAZE_CUDA_TRY(cudaMemcpyAsync(s->seg_off.p, seg.data(), sizeof(uint32_t) * (nq + 1),
                                           cudaMemcpyHostToDevice, s->stream));
            BLAZE_CUDA_TRY(cudaMemcpyAsync(s->sel_limit.p, limit.data(), sizeof(int32_t) * nq,
                                           cudaMemcpyHostToDevice, s->stream));
            BLAZE_CUDA_TRY(cudaMemcpyAsync(s->sel_q.p, sel.data(), sizeof(uint32_t) * sel.size(),
                                           cudaMemcpyHostToDevice, s->stream));
            BLAZE_CUDA_TRY(cudaMemsetAsync(s->seg_fill.p, 0, sizeof(uint32_t) * nq, s->stream));
            s->stats.h2d_bytes += sizeof(uint32_t) * (nq + 1) + sizeof(int32_t) * nq + sizeof(uint32_t) * sel.size();
            HitlistArgs ha{};
            ha.groups = s->groups.p;
            ha.n_groups = n_groups;
            ha.seg_off = s->seg_off.p;
            ha.seg_fill = s->seg_fill.p;
            ha.keys = s->seg_keys.p;
            ha.idx = s->seg_idx.p;
            ha.sel_queries = s->sel_q.p;
            ha.limit = s->sel_limit.p;
            BLAZE_CUDA_TRY(launch_hitlist(ha, static_cast<uint32_t>(sel.size()), s->n_sm, s->stream));
            s->stats.kernel_launches += 2;
        }
    }

    // copy back: the kept HSPs and one descriptor per subject list
    const size_t n_out = static_cast<size_t>(c.out_count);
    if ((rc = ensure_pinned(s->h_out, s->h_out_n, n_out)) != BLAZE_OK) return rc;
    if ((rc = ensure_pinned(s->h_groups, s->h_groups_n, n_groups)) != BLAZE_OK) return rc;
    if (n_out) {
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->h_out, s->out.p, sizeof(DevHsp) * n_out, cudaMemcpyDeviceToHost, s->stream));
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->h_groups, s->groups.p, sizeof(GroupDesc) * n_groups,
                                       cudaMemcpyDeviceToHost, s->stream));
        s->stats.d2h_bytes += sizeof(DevHsp) * n_out + sizeof(GroupDesc) * n_groups;
    }
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[3], s->stream));
    BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
    {
        float ms = 0.f;
        BLAZE_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[1], s->ev[2]));
        s->stats.scan_ms = ms;
        BLAZE_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[0], s->ev[3]));
        s->stats.device_ms = ms;
    }
    // the lists by (query, OID); E-values of the kept HSPs (the reap,
    // max_hsps and the hit list already applied on the device)
    std::vector<const GroupDesc *> order_g;
    order_g.reserve(n_groups);
    for (size_t i = 0; i < n_groups; ++i)
        if (s->h_groups[i].n > 0) order_g.push_back(&s->h_groups[i]);
    std::sort(order_g.begin(), order_g.end(), [](const GroupDesc *a, const GroupDesc *b) {
        return a->query != b->query ? a->query < b->query : a->oid < b->oid;
    });
    size_t n_keep = 0;
    for (const GroupDesc *g : order_g) n_keep += g->n;
    if (batched) s->batch_results.reserve(n_keep);
    else s->results.reserve(n_keep);
    for (const GroupDesc *g : order_g) {
        const blaze_params &pg = r.p[g->query];
        for (uint32_t k = 0; k < g->n; ++k) {
            const DevHsp &d = s->h_out[g->first + k];
            blaze_hsp h;
            h.oid = g->oid;
            h.score = d.score;
            h.q_start = d.q_start;
            h.q_end = d.q_end;
            h.s_start = d.s_start;
            h.s_end = d.s_end;
            h.q_gapped_start = d.q_gs;
            h.s_gapped_start = d.s_gs;
            h.evalue = pg.eff_searchsp * pg.K * std::exp(-pg.lambda * static_cast<double>(d.score));
            if (batched) {
                blaze_batch_hsp bh;
                bh.query = g->query;
                bh.reserved = 0;
                bh.hsp = h;
                s->batch_results.push_back(bh);
            } else {
                s->results.push_back(h);
            }
        }
    }
    const uint32_t subjects = static_cast<uint32_t>(order_g.size());
    const size_t n_res = batched ? s->batch_results.size() : s->results.size();
    s->last_init_count = c.init_count;
    s->last_work_count = c.work_count;
    s->last_batched = batched;
    s->last_batch = r.b;
    s->stats.residues_scanned = c.residues;
    s->stats.word_hits = c.word_hits;
    s->stats.ungapped_extensions = c.extensions;
    s->stats.init_hsps = c.init_count;
    s->stats.gapped_extensions = c.gapped_ext;
    s->stats.dp_cells = c.dp_cells;
    s->stats.hsps = n_res;
    s->stats.subjects_with_hsps = subjects;
    if (n_hsps) *n_hsps = n_res;
    return BLAZE_OK;
}

extern "C" int blaze_search_run(blaze_search *s, const blaze_query *q, const blaze_params *p,
                                uint64_t *n_hsps) try {
    if (!s || !q || q->device != s->db->device) return BLAZE_ERR_INVALID_ARG;
    int rc = check_params(p);
    if (rc != BLAZE_OK) return rc;
    if (p->word_threshold != q->threshold) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    RunSpec r;
    r.q = q;
    r.p = p;
    rc = run_search(s, r, n_hsps);
    s->stats.h2d_bytes += q->upload_bytes;
    return rc;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_run_batch(blaze_search *s, const blaze_batch *b, const blaze_params *params,
                                      uint64_t *n_hsps) try {
    if (!s || !b || !params || b->device != s->db->device || b->n == 0) return BLAZE_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < b->n; ++i) {
        int rc = check_params(&params[i]);
        if (rc != BLAZE_OK) return rc;
        const blaze_params &a = params[0], &c = params[i];
        if (c.word_threshold != b->threshold || c.window != a.window || c.ungapped_xdrop != a.ungapped_xdrop ||
            c.gap_open != a.gap_open || c.gap_extend != a.gap_extend || c.gapped_xdrop != a.gapped_xdrop)
            return BLAZE_ERR_INVALID_ARG;
    }
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    RunSpec r;
    r.b = b;
    r.p = params;
    int rc = run_search(s, r, n_hsps);
    s->stats.h2d_bytes += b->upload_bytes;
    return rc;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_batch_results(const blaze_search *s, blaze_batch_hsp *out, uint64_t capacity,
                                          uint64_t *n_hsps) try {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    if (n_hsps) *n_hsps = s->batch_results.size();
    if (capacity < s->batch_results.size()) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (!s->batch_results.empty()) {
        if (!out) return BLAZE_ERR_INVALID_ARG;
        std::memcpy(out, s->batch_results.data(), sizeof(blaze_batch_hsp) * s->batch_results.size());
    }
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_set_tuning(blaze_search *s, const blaze_tuning *t) try {
    if (!s || !t) return BLAZE_ERR_INVALID_ARG;
    if (t->stage_bytes > 16384 || t->max_warps_per_block > static_cast<uint32_t>(kScanMaxWarpsPerBlock))
        return BLAZE_ERR_LIMIT;
    if (t->launch_mode > 2 || t->batch_launch > 2) return BLAZE_ERR_INVALID_ARG;
    s->launch_mode = t->launch_mode;
    s->batch_launch = t->batch_launch;
    s->stage_bytes = t->stage_bytes ? t->stage_bytes : kScanStageBytes;
    s->tile_residues = t->tile_residues;
    s->max_warps = t->max_warps_per_block;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_results(const blaze_search *s, blaze_hsp *out, uint64_t capacity,
                                    uint64_t *n_hsps) try {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    if (n_hsps) *n_hsps = s->results.size();
    if (capacity < s->results.size()) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (!s->results.empty()) {
        if (!out) return BLAZE_ERR_INVALID_ARG;
        std::memcpy(out, s->results.data(), sizeof(blaze_hsp) * s->results.size());
    }
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_stats(const blaze_search *s, blaze_stats *out) {
    if (!s || !out) return BLAZE_ERR_INVALID_ARG;
    *out = s->stats;
    return BLAZE_OK;
}

extern "C" int blaze_search_init_hits(blaze_search *s, blaze_init_hit *out, uint64_t capacity,
                                      uint64_t *n_hits) try {
    if (!s || s->last_batched) return BLAZE_ERR_INVALID_ARG;  // single-query runs only
    const size_t n_init = static_cast<size_t>(s->last_init_count);
    const size_t n_work = static_cast<size_t>(s->last_work_count);
    if (n_hits) *n_hits = n_init;
    if (capacity < n_init) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (n_init == 0) return BLAZE_OK;
    if (!out) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    std::vector<InitHit> hits(n_init);
    std::vector<WorkItem> work(n_work);
    BLAZE_CUDA_TRY(cudaMemcpy(hits.data(), s->init_out.p, sizeof(InitHit) * n_init, cudaMemcpyDeviceToHost));
    BLAZE_CUDA_TRY(cudaMemcpy(work.data(), s->work.p, sizeof(WorkItem) * n_work, cudaMemcpyDeviceToHost));
    std::sort(work.begin(), work.end(), [&](const WorkItem &a, const WorkItem &b) {
        return s->db->oid_of[a.subject] < s->db->oid_of[b.subject];
    });
    size_t k = 0;
    for (const WorkItem &w : work) {
        std::vector<InitHit> sub(hits.begin() + w.first, hits.begin() + w.first + w.n_init);
        std::sort(sub.begin(), sub.end(), [](const InitHit &x, const InitHit &y) {
            if (x.score != y.score) return x.score > y.score;
            if (x.s_trig != y.s_trig) return x.s_trig < y.s_trig;
            return x.q_trig < y.q_trig;
        });
        for (const InitHit &h : sub) {
            blaze_init_hit &o = out[k++];
            o.oid = s->db->oid_of[w.subject];
            o.q_start = h.q_start;
            o.s_start = h.s_start;
            o.length = h.len;
            o.score = h.score;
            o.q_trigger = h.q_trig;
            o.s_trigger = h.s_trig;
        }
    }
    if (n_hits) *n_hits = k;
    return k == n_init ? BLAZE_OK : BLAZE_ERR_INTERNAL;
} BLAZE_ABI_CATCH

// One call with host buffers: the query's tables go into buffers the search
// context keeps (grown on demand), copied from pinned staging on the
// search's stream ahead of the kernels -- no allocation and no device-wide
// synchronisation per query once warm.
extern "C" int blaze_prelim_search(blaze_search *s, const uint8_t *query, int32_t length,
                                   const blaze_params *p, blaze_hsp *out, uint64_t capacity,
                                   uint64_t *n_hsps) try {
    if (!s || !p || !query || length <= 0) return BLAZE_ERR_INVALID_ARG;
    if (length > kMaxQueryLength) return BLAZE_ERR_LIMIT;
    if (!valid_residues(query, static_cast<uint64_t>(length))) return BLAZE_ERR_INVALID_ARG;
    int rc = check_params(p);
    if (rc != BLAZE_OK) return rc;
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    QueryTables t;
    if ((rc = query_tables(query, length, p->word_threshold, t)) != BLAZE_OK) return rc;
    // pinned staging: residues (+ 64 zero bytes), cell_start, packed cells, presence, hit lists
    const size_t b_q = (static_cast<size_t>(length) + 64 + 15) & ~size_t{15};
    const size_t b_cs = sizeof(uint32_t) * (kWords + 1), b_pack = sizeof(uint32_t) * kWords;
    const size_t b_pres = sizeof(uint32_t) * kPresenceWords, b_off = sizeof(uint16_t) * t.n_off;
    const size_t o_cs = b_q, o_pack = (o_cs + b_cs + 15) & ~size_t{15}, o_pres = o_pack + b_pack,
                 o_off = (o_pres + b_pres + 15) & ~size_t{15};
    if ((rc = ensure_pinned(s->h_stage, s->h_stage_n, o_off + b_off)) != BLAZE_OK) return rc;
    unsigned char *h = s->h_stage;
    std::memcpy(h, query, length);
    std::memset(h + length, 0, b_q - static_cast<size_t>(length));
    std::memcpy(h + o_cs, t.cs.data(), b_cs);
    std::memcpy(h + o_pack, t.pack.data(), b_pack);
    std::memcpy(h + o_pres, t.pres.data(), b_pres);
    if (b_off) std::memcpy(h + o_off, t.offs, b_off);
    if ((rc = s->qt_res.ensure(b_q)) != BLAZE_OK) return rc;
    if ((rc = s->qt_cs.ensure(kWords + 1)) != BLAZE_OK) return rc;
    if ((rc = s->qt_pack.ensure(kWords)) != BLAZE_OK) return rc;
    if ((rc = s->qt_pres.ensure(kPresenceWords)) != BLAZE_OK) return rc;
    if ((rc = s->qt_off.ensure(std::max<uint32_t>(t.n_off, 1))) != BLAZE_OK) return rc;
    BLAZE_CUDA_TRY(cudaMemcpyAsync(s->qt_res.p, h, b_q, cudaMemcpyHostToDevice, s->stream));
    BLAZE_CUDA_TRY(cudaMemcpyAsync(s->qt_cs.p, h + o_cs, b_cs, cudaMemcpyHostToDevice, s->stream));
    BLAZE_CUDA_TRY(cudaMemcpyAsync(s->qt_pack.p, h + o_pack, b_pack, cudaMemcpyHostToDevice, s->stream));
    BLAZE_CUDA_TRY(cudaMemcpyAsync(s->qt_pres.p, h + o_pres, b_pres, cudaMemcpyHostToDevice, s->stream));
    if (b_off) BLAZE_CUDA_TRY(cudaMemcpyAsync(s->qt_off.p, h + o_off, b_off, cudaMemcpyHostToDevice, s->stream));
    blaze_query q;  // views of the search's buffers; not freed
    q.device = s->db->device;
    q.qlen = length;
    q.threshold = p->word_threshold;
    q.n_off = t.n_off;
    q.upload_bytes = query_upload_bytes(length, t.n_off);
    q.d_q = s->qt_res.p;
    q.d_cell_start = s->qt_cs.p;
    q.d_cell_pack = s->qt_pack.p;
    q.d_presence = s->qt_pres.p;
    q.d_cell_off = s->qt_off.p;
    RunSpec r;
    r.q = &q;
    r.p = p;
    rc = run_search(s, r, n_hsps);  // synchronises the stream before it returns
    s->stats.h2d_bytes += q.upload_bytes;
    if (rc != BLAZE_OK) return rc;
    return blaze_search_results(s, out, capacity, n_hsps);
} BLAZE_ABI_CATCH
