// api.cu -- C ABI of libblaze103: resident database, query tables, and the
// search driver that runs the two device stages and finishes each subject's
// HSP list (E-values, preliminary E-value reap, OID order) on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"

using namespace blaze;

namespace {
thread_local cudaError_t g_last_cuda = cudaSuccess;
constexpr uint32_t kMaxSubjectLength = (1u << 28) - 64;  // diagonal table encoding limit
constexpr int32_t kMaxQueryLength = 32000;                // diagonal table must fit shared memory
constexpr uint32_t kInitialScratchCap = 1024;             // init hits per subject before a rerun
}  // namespace

void last_cuda_error(cudaError_t e) { g_last_cuda = e; }

extern "C" const char *blaze_last_cuda_error(void) { return cudaGetErrorString(g_last_cuda); }

struct blaze_db {
    int device = 0;
    uint8_t *d_res = nullptr;
    uint64_t *d_off = nullptr;
    uint64_t total = 0;
    uint32_t n = 0;
    uint32_t max_len = 0;
    std::vector<uint32_t> oid_of;  // sorted index -> OID
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
    DevCounters *d_cnt = nullptr;
    DevCounters *h_cnt = nullptr;  // pinned
    DevHsp *h_out = nullptr;       // pinned
    size_t h_out_n = 0;
    int gapped_blocks = 0;
    std::vector<blaze_hsp> results;
    blaze_stats stats{};
    unsigned long long last_init_count = 0, last_work_count = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

static bool valid_residues(const uint8_t *r, uint64_t n) {
    uint8_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) bad |= static_cast<uint8_t>(r[i] == 0) | static_cast<uint8_t>(r[i] >= kAlphabet);
    return bad == 0;
}

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
                               uint32_t n_subjects, blaze_db **out) {
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
        if (e != cudaSuccess) {
            last_cuda_error(e);
            rc = BLAZE_ERR_CUDA;
        }
    } while (false);
    if (rc != BLAZE_OK) {
        blaze_db_free(db);
        return rc;
    }
    *out = db;
    return BLAZE_OK;
}

extern "C" int blaze_db_free(blaze_db *db) {
    if (!db) return BLAZE_OK;
    cudaSetDevice(db->device);
    if (db->d_res) cudaFree(db->d_res);
    if (db->d_off) cudaFree(db->d_off);
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

extern "C" int blaze_query_create(const blaze_db *db, const uint8_t *query, int32_t length,
                                  int32_t word_threshold, blaze_query **out) {
    if (!db || !query || !out || length <= 0) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    if (length > kMaxQueryLength) return BLAZE_ERR_LIMIT;
    if (!valid_residues(query, static_cast<uint64_t>(length))) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(db->device));
    std::vector<uint32_t> cs(kWords + 1);
    uint16_t *offs = nullptr;
    uint32_t n_off = 0;
    int rc = build_lookup(query, length, word_threshold, cs.data(), &offs, &n_off);
    if (rc != BLAZE_OK) return rc;
    auto *q = new blaze_query();
    q->device = db->device;
    q->qlen = length;
    q->threshold = word_threshold;
    q->n_off = n_off;
    cudaError_t e = cudaMalloc(&q->d_q, static_cast<size_t>(length) + 64);
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_start, sizeof(uint32_t) * (kWords + 1));
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_off, sizeof(uint16_t) * std::max<uint32_t>(n_off, 1));
    // packed cells (start << 8 | count, 255 = look at cell_start) and the
    // word-presence bitset of the scan kernel
    std::vector<uint32_t> pack(kWords), pres(kPresenceWords, 0u);
    for (int w = 0; w < kWords; ++w) {
        const uint32_t cnt = cs[w + 1] - cs[w];
        pack[w] = (cs[w] << 8) | std::min<uint32_t>(cnt, 255u);
        if (cnt) pres[w >> 5] |= 1u << (w & 31);
    }
    if (e == cudaSuccess) e = cudaMalloc(&q->d_cell_pack, sizeof(uint32_t) * kWords);
    if (e == cudaSuccess) e = cudaMalloc(&q->d_presence, sizeof(uint32_t) * kPresenceWords);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_cell_pack, pack.data(), sizeof(uint32_t) * kWords, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_presence, pres.data(), sizeof(uint32_t) * kPresenceWords, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_q, query, length, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(q->d_q + length, 0, 64);
    if (e == cudaSuccess) e = cudaMemcpy(q->d_cell_start, cs.data(), sizeof(uint32_t) * (kWords + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_off) e = cudaMemcpy(q->d_cell_off, offs, sizeof(uint16_t) * n_off, cudaMemcpyHostToDevice);
    std::free(offs);
    q->upload_bytes = static_cast<uint64_t>(length) + sizeof(uint32_t) * (2 * kWords + 1 + kPresenceWords) +
                      sizeof(uint16_t) * n_off;
    if (e != cudaSuccess) {
        last_cuda_error(e);
        blaze_query_free(q);
        return e == cudaErrorMemoryAllocation ? BLAZE_ERR_OUT_OF_MEMORY : BLAZE_ERR_CUDA;
    }
    *out = q;
    return BLAZE_OK;
}

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

extern "C" int blaze_search_create(blaze_db *db, blaze_search **out) {
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
    s->out_cap = std::max<unsigned long long>(1ull << 20, db->n / 16);
    // Starting capacities can be lowered (e.g. to exercise the grow-and-repeat
    // path); they grow on demand either way.
    if (const char *v = std::getenv("BLAZE_INITIAL_SCRATCH_CAP")) s->scratch_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_INIT_CAP")) s->init_cap = std::max(1, std::atoi(v));
    if (const char *v = std::getenv("BLAZE_INITIAL_OUT_CAP")) s->out_cap = std::max(1, std::atoi(v));
    *out = s;
    return BLAZE_OK;
}

extern "C" int blaze_search_free(blaze_search *s) {
    if (!s) return BLAZE_OK;
    cudaSetDevice(s->db->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->scratch.release();
    s->init_out.release();
    s->sorted.release();
    s->work.release();
    s->saved.release();
    s->out.release();
    s->dp.release();
    if (s->d_cnt) cudaFree(s->d_cnt);
    if (s->h_cnt) cudaFreeHost(s->h_cnt);
    if (s->h_out) cudaFreeHost(s->h_out);
    for (cudaEvent_t ev : s->ev)
        if (ev) cudaEventDestroy(ev);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return BLAZE_OK;
}

static int check_params(const blaze_params *p) {
    if (!p) return BLAZE_ERR_INVALID_ARG;
    if (p->window <= 0 || p->window > (1 << 20) || p->ungapped_xdrop <= 0 || p->gap_open < 0 ||
        p->gap_extend <= 0 || p->gapped_xdrop <= 0 || p->gapped_cutoff <= 0 || p->ungapped_cutoff <= 0)
        return BLAZE_ERR_INVALID_ARG;
    return BLAZE_OK;
}

// One pass of both stages; fills s->h_cnt.
static int run_pass(blaze_search *s, const blaze_query *q, const blaze_params *p, const ScanLayout &lay,
                    int scan_blocks) {
    const int warps_per_block = lay.warps_per_block;
    blaze_db *db = s->db;
    const size_t scan_warps = static_cast<size_t>(scan_blocks) * warps_per_block;
    const size_t gapped_warps = static_cast<size_t>(s->gapped_blocks) * kGappedWarpsPerBlock;
    int rc;
    if ((rc = s->scratch.ensure(scan_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->sorted.ensure(gapped_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->saved.ensure(gapped_warps * s->scratch_cap)) != BLAZE_OK) return rc;
    if ((rc = s->init_out.ensure(s->init_cap)) != BLAZE_OK) return rc;
    if ((rc = s->work.ensure(std::max<uint32_t>(db->n, 1))) != BLAZE_OK) return rc;
    if ((rc = s->out.ensure(s->out_cap)) != BLAZE_OK) return rc;
    const size_t dp_stride = static_cast<size_t>(std::max<uint32_t>(db->max_len, 1)) + 2;
    if ((rc = s->dp.ensure(gapped_warps * 2 * dp_stride)) != BLAZE_OK) return rc;

    BLAZE_CUDA_TRY(cudaMemsetAsync(s->d_cnt, 0, sizeof(DevCounters), s->stream));
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[1], s->stream));
    ScanArgs sa{};
    sa.res = db->d_res;
    sa.off = db->d_off;
    sa.n_subj = db->n;
    sa.q = q->d_q;
    sa.qlen = q->qlen;
    sa.cell_start = q->d_cell_start;
    sa.cell_pack = q->d_cell_pack;
    sa.presence = q->d_presence;
    sa.cell_off = q->d_cell_off;
    sa.window = p->window;
    sa.xdrop = p->ungapped_xdrop;
    sa.cutoff = p->ungapped_cutoff;
    sa.diag_entries = lay.diag_entries;
    sa.diag_magic = lay.diag_magic;
    sa.diag_bytes = lay.diag_bytes;
    sa.stage_bytes = lay.stage_bytes;
    sa.query_smem_bytes = lay.query_smem_bytes;
    sa.warp_smem_bytes = lay.warp_smem_bytes;
    sa.scratch = s->scratch.p;
    sa.scratch_cap = s->scratch_cap;
    sa.init_out = s->init_out.p;
    sa.init_cap = s->init_cap;
    sa.work = s->work.p;
    sa.work_cap = s->work.n;
    sa.cnt = s->d_cnt;
    BLAZE_CUDA_TRY(launch_scan(sa, scan_blocks, warps_per_block, lay.smem_bytes, s->stream));
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[2], s->stream));

    GappedArgs ga{};
    ga.res = db->d_res;
    ga.off = db->d_off;
    ga.q = q->d_q;
    ga.qlen = q->qlen;
    ga.init_in = s->init_out.p;
    ga.work = s->work.p;
    ga.work_cap = s->work.n;
    ga.sorted = s->sorted.p;
    ga.saved = s->saved.p;
    ga.cap = s->scratch_cap;
    ga.dp = s->dp.p;
    ga.dp_stride = static_cast<uint32_t>(dp_stride);
    ga.gap_open = p->gap_open;
    ga.gap_extend = p->gap_extend;
    ga.xdrop = p->gapped_xdrop;
    ga.cutoff = p->gapped_cutoff;
    ga.out = s->out.p;
    ga.out_cap = s->out_cap;
    ga.cnt = s->d_cnt;
    BLAZE_CUDA_TRY(launch_gapped(ga, s->gapped_blocks, s->stream));
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[3], s->stream));
    s->stats.kernel_launches += 2;
    s->stats.d2h_bytes += sizeof(DevCounters);
    BLAZE_CUDA_TRY(cudaMemcpyAsync(s->h_cnt, s->d_cnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, s->stream));
    BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return BLAZE_OK;
}

extern "C" int blaze_search_run(blaze_search *s, const blaze_query *q, const blaze_params *p,
                                uint64_t *n_hsps) {
    if (!s || !q || q->device != s->db->device) return BLAZE_ERR_INVALID_ARG;
    int rc = check_params(p);
    if (rc != BLAZE_OK) return rc;
    if (p->word_threshold != q->threshold) return BLAZE_ERR_INVALID_ARG;
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    s->results.clear();
    s->stats = blaze_stats{};
    s->stats.h2d_bytes = q->upload_bytes;
    if (n_hsps) *n_hsps = 0;

    constexpr size_t kSmemBudget = 220 * 1024;
    const bool qsmem = q->qlen <= kQuerySmemMax;
    const ScanLayout lay = scan_layout(q->qlen, p->window, kScanStageBytes, kSmemBudget,
                                       scan_max_warps_by_registers(qsmem));
    if (lay.smem_bytes > 227 * 1024) return BLAZE_ERR_LIMIT;
    int per_sm = 0;
    BLAZE_CUDA_TRY(scan_occupancy(lay.query_smem_bytes != 0, lay.warps_per_block, lay.smem_bytes, &per_sm));
    if (per_sm < 1) return BLAZE_ERR_LIMIT;
    const int scan_blocks = s->n_sm * per_sm;

    DevCounters c{};
    BLAZE_CUDA_TRY(cudaEventRecord(s->ev[0], s->stream));
    for (int attempt = 0;; ++attempt) {
        if ((rc = run_pass(s, q, p, lay, scan_blocks)) != BLAZE_OK) return rc;
        c = *s->h_cnt;
        {
            float ms = 0.f;
            BLAZE_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[2], s->ev[3]));
            s->stats.gapped_ms = ms;
        }
        if (c.flags & kFlagBadState) return BLAZE_ERR_INTERNAL;
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
        if (c.flags & kFlagWorkArrayFull) return BLAZE_ERR_INTERNAL;  // one item per subject at most
        if (!again) break;
        if (attempt >= 6) return BLAZE_ERR_INTERNAL;
        s->stats.reruns++;
    }

    // copy back and finish on the host
    const size_t n_out = static_cast<size_t>(c.out_count);
    if (n_out > s->h_out_n) {
        if (s->h_out) cudaFreeHost(s->h_out);
        s->h_out = nullptr;
        s->h_out_n = 0;
        BLAZE_CUDA_TRY(cudaMallocHost(&s->h_out, sizeof(DevHsp) * n_out));
        s->h_out_n = n_out;
    }
    if (n_out) {
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->h_out, s->out.p, sizeof(DevHsp) * n_out, cudaMemcpyDeviceToHost, s->stream));
        s->stats.d2h_bytes += sizeof(DevHsp) * n_out;
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
    // groups: each subject's HSPs are contiguous and already in final order
    struct Group { uint32_t oid; size_t first, n; };
    std::vector<Group> groups;
    for (size_t i = 0; i < n_out;) {
        size_t j = i + 1;
        while (j < n_out && s->h_out[j].subject == s->h_out[i].subject) ++j;
        groups.push_back({s->db->oid_of[s->h_out[i].subject], i, j - i});
        i = j;
    }
    std::sort(groups.begin(), groups.end(), [](const Group &a, const Group &b) { return a.oid < b.oid; });
    s->results.reserve(n_out);
    uint32_t subjects = 0;
    for (const Group &g : groups) {
        size_t kept = 0;
        for (size_t k = 0; k < g.n; ++k) {
            const DevHsp &d = s->h_out[g.first + k];
            blaze_hsp h;
            h.oid = g.oid;
            h.score = d.score;
            h.q_start = d.q_start;
            h.q_end = d.q_end;
            h.s_start = d.s_start;
            h.s_end = d.s_end;
            h.q_gapped_start = d.q_gs;
            h.s_gapped_start = d.s_gs;
            h.evalue = p->eff_searchsp * p->K * std::exp(-p->lambda * static_cast<double>(d.score));
            if (h.evalue > p->prelim_evalue) continue;  // preliminary E-value reap
            s->results.push_back(h);
            ++kept;
        }
        subjects += kept > 0;
    }
    s->last_init_count = c.init_count;
    s->last_work_count = c.work_count;
    s->stats.residues_scanned = c.residues;
    s->stats.word_hits = c.word_hits;
    s->stats.ungapped_extensions = c.extensions;
    s->stats.init_hsps = c.init_count;
    s->stats.gapped_extensions = c.gapped_ext;
    s->stats.dp_cells = c.dp_cells;
    s->stats.hsps = s->results.size();
    s->stats.subjects_with_hsps = subjects;
    if (n_hsps) *n_hsps = s->results.size();
    return BLAZE_OK;
}

extern "C" int blaze_search_results(const blaze_search *s, blaze_hsp *out, uint64_t capacity,
                                    uint64_t *n_hsps) {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    if (n_hsps) *n_hsps = s->results.size();
    if (capacity < s->results.size()) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (!s->results.empty()) {
        if (!out) return BLAZE_ERR_INVALID_ARG;
        std::memcpy(out, s->results.data(), sizeof(blaze_hsp) * s->results.size());
    }
    return BLAZE_OK;
}

extern "C" int blaze_search_stats(const blaze_search *s, blaze_stats *out) {
    if (!s || !out) return BLAZE_ERR_INVALID_ARG;
    *out = s->stats;
    return BLAZE_OK;
}

extern "C" int blaze_search_init_hits(blaze_search *s, blaze_init_hit *out, uint64_t capacity,
                                      uint64_t *n_hits) {
    if (!s) return BLAZE_ERR_INVALID_ARG;
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
}

extern "C" int blaze_prelim_search(blaze_search *s, const uint8_t *query, int32_t length,
                                   const blaze_params *p, blaze_hsp *out, uint64_t capacity,
                                   uint64_t *n_hsps) {
    if (!s || !p) return BLAZE_ERR_INVALID_ARG;
    blaze_query *q = nullptr;
    int rc = blaze_query_create(s->db, query, length, p->word_threshold, &q);
    if (rc != BLAZE_OK) return rc;
    rc = blaze_search_run(s, q, p, n_hsps);
    blaze_query_free(q);
    if (rc != BLAZE_OK) return rc;
    return blaze_search_results(s, out, capacity, n_hsps);
}
