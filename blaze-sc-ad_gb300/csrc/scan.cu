// scan.cu -- word finder, two-hit seeding and ungapped X-drop extension of
// the BLASTP preliminary search on GB300 (sm_103a). Integer work only.
//
// One warp per subject; persistent warps pull subjects, longest first, from a
// device cursor. Per block in shared memory: the BLOSUM62 matrix (int8), the
// query's word-presence bitset and, for queries up to kQuerySmemMax, the
// query residues. Per warp: the diagonal table, the deferred-hit and seed
// queues and a staging buffer that holds the whole subject when it fits, so
// the word scan and the extensions read shared memory instead of making
// dependent global loads.
//
// Reference counterpart: gpuBLAZE_full (BLAZE_gpu/gpuBLAZE.cu:885-1252), which
// is a filter; this kernel produces the exact ungapped HSPs of the
// sequential algorithm.
#include <cstdint>

#include "common.cuh"

namespace blaze {
namespace {

__device__ const int8_t g_blosum8[kAlphabet * kAlphabet] = {
#include "blosum62_i8.inc"
};

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kFlagBit = 0x80000000u;  // diagonal: an extension ran right
constexpr uint32_t kPendBit = 0x40000000u;  // diagonal: a seed waits for its extension
constexpr uint32_t kValMask = 0x3fffffffu;
constexpr uint32_t kBaseReset = 1u << 28;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// idx mod L for idx < 2^32, with magic = floor(2^32 / L) + 1: the estimated
// quotient is the true one or one more.
__device__ __forceinline__ uint32_t fast_mod(uint32_t idx, uint32_t L, uint32_t magic) {
    const uint32_t qt = __umulhi(idx, magic);
    const int32_t r = static_cast<int32_t>(idx - qt * L);
    return static_cast<uint32_t>(r < 0 ? r + static_cast<int32_t>(L) : r);
}

// ------------------------------------------------------------------------
// Ungapped extension (scalar, one lane per seed); q and s are generic
// pointers (shared memory when staged, global otherwise).

__device__ __forceinline__ int32_t extend_left(const uint8_t *q, const uint8_t *s, int32_t q_off,
                                               int32_t s_off, int32_t xdrop, const int8_t *mat,
                                               int32_t *length) {
    const int32_t n = min(s_off, q_off);
    int32_t best_k = -1, score = 0, maxscore = 0;
    const uint8_t *qq = q + q_off, *ss = s + s_off;
    for (int32_t k = 0; k <= n; ++k) {
        score += mat[qq[-k] * kAlphabet + ss[-k]];
        if (score > maxscore) {
            maxscore = score;
            best_k = k;
        }
        if (maxscore - score >= xdrop) break;
    }
    *length = best_k + 1;
    return maxscore;
}

__device__ __forceinline__ int32_t extend_right(const uint8_t *q, int32_t qlen, const uint8_t *s,
                                                int32_t slen, int32_t q_off, int32_t s_off,
                                                int32_t xdrop, int32_t maxscore, const int8_t *mat,
                                                int32_t *length, int32_t *s_last_off) {
    const int32_t n = min(slen - s_off, qlen - q_off);
    int32_t best_i = -1, score = maxscore, i;
    const uint8_t *qq = q + q_off, *ss = s + s_off;
    for (i = 0; i < n; ++i) {
        score += mat[qq[i] * kAlphabet + ss[i]];
        if (score > maxscore) {
            maxscore = score;
            best_i = i;
        }
        if (score <= 0 || maxscore - score >= xdrop) break;
    }
    *length = best_i + 1;
    *s_last_off = s_off + i;
    return maxscore;
}

// Two-hit extension from the second hit (q_off, s_off); s_left_off is the
// end of the first hit (gpuBLAZE.cu:1096-1152 is the warp-parallel form).
__device__ __forceinline__ int32_t extend_two_hit(const uint8_t *q, int32_t qlen, const uint8_t *s,
                                                  int32_t slen, int32_t s_left_off, int32_t s_off,
                                                  int32_t q_off, int32_t xdrop, const int8_t *mat,
                                                  int32_t *hsp_q, int32_t *hsp_s, int32_t *hsp_len,
                                                  int32_t *right_extend, int32_t *s_last_off) {
    int32_t score = 0, left_score = 0, right_d = 0, left_d = 0, right_score = 0;
#pragma unroll
    for (int32_t i = 0; i < kWordSize; ++i) {
        score += mat[q[q_off + i] * kAlphabet + s[s_off + i]];
        if (score > left_score) {
            left_score = score;
            right_d = i + 1;
        }
    }
    const int32_t q_right = q_off + right_d, s_right = s_off + right_d;
    left_score = extend_left(q, s, q_right - 1, s_right - 1, xdrop, mat, &left_d);
    right_d = 0;
    *right_extend = 0;
    *s_last_off = s_right;
    if (left_d >= s_right - s_left_off) {
        *right_extend = 1;
        right_score = extend_right(q, qlen, s, slen, q_right, s_right, xdrop, left_score, mat,
                                   &right_d, s_last_off);
    }
    *hsp_q = q_right - left_d;
    *hsp_s = s_right - left_d;
    *hsp_len = left_d + right_d;
    return max(left_score, right_score);
}

// ------------------------------------------------------------------------
// Word finder state of one warp. The diagonal table holds, per diagonal
// (s - q) mod L, either the last recorded hit (biased by window and by a
// running base so the table never needs clearing between subjects), the same
// with kFlagBit after a right extension, or kPendBit | seed slot while that
// diagonal's extension is queued. With L >= qlen + window two diagonals that
// share an entry never both matter: all hits of the later one come more than
// `window` positions after every hit of the earlier one and after the end of
// any extension on it.

struct WarpFinder {
    uint32_t *diag;
    uint2 *defer;  // two buffers of kDeferCap deferred hits {s, q}, arrival order
    int4 *seeds;   // {q, s, s_left_off, table index}
    int n_defer, n_seed, sel;
    uint32_t base;
    uint32_t n_init;
    const uint8_t *sub;  // generic: staged copy or global
    const uint8_t *q;    // generic: shared copy or global
    int32_t slen;
    InitHit *scratch;
    unsigned long long extensions;
};

enum : int { kActNone = 0, kActSet = 1, kActSeed = 2, kActDefer = 3 };

// Runs up to 32 hits (one per lane, lanes in hit order) through the two-hit
// logic. Hits on the same diagonal are taken in lane order; a hit whose
// diagonal waits on an extension is appended to the deferred list.
__device__ __forceinline__ void process_batch(WarpFinder &wf, const ScanArgs &a, bool valid,
                                              int32_t s, int32_t q) {
    if (__ballot_sync(kFull, valid) == 0) return;
    const uint32_t d = fast_mod(static_cast<uint32_t>(s - q + a.qlen), a.diag_entries, a.diag_magic);
    const unsigned lt = lanemask_lt();
    const unsigned peers = __match_any_sync(kFull, valid ? d : 0xffffffffu);
    const unsigned rank = valid ? __popc(peers & lt) : 0u;
    const unsigned max_rank = __reduce_max_sync(kFull, rank);
    const uint32_t here = static_cast<uint32_t>(s + a.window) + wf.base;  // s, biased
    for (unsigned r = 0; r <= max_rank; ++r) {
        const bool mine = valid && rank == r;
        const uint32_t e = mine ? wf.diag[d] : 0u;
        const bool pend = (e & kPendBit) != 0u;
        const bool flag = (e & kFlagBit) != 0u;
        const int32_t last = static_cast<int32_t>(e & kValMask) - a.window - static_cast<int32_t>(wf.base);
        const int32_t diff = s - last;
        // flag set: hits inside the last extension are skipped, the first one
        // past it starts over; otherwise a hit far from the last one starts
        // over, one at distance [wordsize, window) triggers an extension, and
        // an overlapping one is ignored
        const bool defer = mine && pend;
        const bool seed = mine && !pend && !flag && diff >= kWordSize && diff < a.window;
        const bool set = mine && !pend && (flag ? s >= last : diff >= a.window);
        if (set) wf.diag[d] = here;
        const unsigned dm = __ballot_sync(kFull, defer);
        const unsigned sm = __ballot_sync(kFull, seed);
        if ((dm | sm) != 0u) {
            if (defer)
                wf.defer[wf.sel * kDeferCap + wf.n_defer + __popc(dm & lt)] =
                    make_uint2(static_cast<uint32_t>(s), static_cast<uint32_t>(q));
            if (seed) {
                const int slot = wf.n_seed + __popc(sm & lt);
                wf.seeds[slot] = make_int4(q, s, last + kWordSize, static_cast<int32_t>(d));
                wf.diag[d] = kPendBit | static_cast<uint32_t>(slot);
            }
            wf.n_defer += __popc(dm);
            wf.n_seed += __popc(sm);
        }
        __syncwarp();
    }
}

// Extends every queued seed (one lane each), settles their diagonals, keeps
// those reaching the ungapped cutoff, then replays the deferred hits; repeats
// until no seed and no deferred hit is left. Each replay is shorter than the
// list it replays whenever it queues a seed, so the loop ends.
__device__ void flush(WarpFinder &wf, const ScanArgs &a, const int8_t *mat) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    while (wf.n_seed > 0 || wf.n_defer > 0) {
        for (int c = 0; c < wf.n_seed; c += 32) {
            const int i = c + lane;
            bool pass = false;
            int32_t hq = 0, hs = 0, hl = 0, score = 0;
            int4 sd = make_int4(0, 0, 0, 0);
            if (i < wf.n_seed) {
                sd = wf.seeds[i];
                int32_t rext, slast;
                score = extend_two_hit(wf.q, a.qlen, wf.sub, wf.slen, sd.z, sd.y, sd.x, a.xdrop, mat,
                                       &hq, &hs, &hl, &rext, &slast);
                wf.diag[sd.w] = rext ? (kFlagBit | (static_cast<uint32_t>(slast - (kWordSize - 1) + a.window) + wf.base))
                                     : (static_cast<uint32_t>(sd.y + a.window) + wf.base);
                pass = score >= a.cutoff;
            }
            const unsigned pm = __ballot_sync(kFull, pass);
            if (pass) {
                const uint32_t pos = wf.n_init + __popc(pm & lt);
                if (pos < a.scratch_cap) {
                    InitHit h;
                    h.q_start = hq;
                    h.s_start = hs;
                    h.len = hl;
                    h.score = score;
                    h.q_trig = sd.x;
                    h.s_trig = sd.y;
                    wf.scratch[pos] = h;
                }
            }
            wf.n_init += __popc(pm);
        }
        wf.extensions += static_cast<unsigned long long>(wf.n_seed);
        wf.n_seed = 0;
        __syncwarp();
        if (wf.n_defer > 0) {
            const int old = wf.sel, n_old = wf.n_defer;
            wf.sel ^= 1;
            wf.n_defer = 0;
            for (int c = 0; c < n_old; c += 32) {
                const int i = c + lane;
                const bool v = i < n_old;
                const uint2 h = v ? wf.defer[old * kDeferCap + i] : make_uint2(0u, 0u);
                process_batch(wf, a, v, static_cast<int32_t>(h.x), static_cast<int32_t>(h.y));
            }
        }
    }
}

__global__ void __launch_bounds__(kScanMaxWarpsPerBlock * 32, 1)
scan_kernel(const ScanArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int8_t *mat = reinterpret_cast<int8_t *>(smem);
    uint32_t *presence = reinterpret_cast<uint32_t *>(smem + kScanMatBytes);
    uint8_t *qsm = smem + kScanMatBytes + kScanPresenceBytes;
    unsigned char *mine = smem + kScanMatBytes + kScanPresenceBytes + a.query_smem_bytes +
                          static_cast<size_t>(warp) * a.warp_smem_bytes;
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x) mat[i] = g_blosum8[i];
    for (int i = threadIdx.x; i < kPresenceWords; i += blockDim.x) presence[i] = a.presence[i];
    if (a.query_smem_bytes)
        for (int i = threadIdx.x; i < a.qlen; i += blockDim.x) qsm[i] = a.q[i];

    WarpFinder wf;
    wf.diag = reinterpret_cast<uint32_t *>(mine);
    wf.defer = reinterpret_cast<uint2 *>(mine + a.diag_bytes);
    wf.seeds = reinterpret_cast<int4 *>(wf.defer + 2 * kDeferCap);
    uint8_t *stage = reinterpret_cast<uint8_t *>(wf.seeds + kSeedCap);
    wf.n_defer = wf.n_seed = wf.sel = 0;
    wf.base = 0;
    wf.extensions = 0;
    wf.q = a.query_smem_bytes ? qsm : a.q;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    wf.scratch = a.scratch + gwarp * a.scratch_cap;
    for (uint32_t i = lane; i < a.diag_entries; i += 32) wf.diag[i] = 0;
    __syncthreads();

    unsigned long long word_hits = 0, residues = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_scan, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= a.n_subj) break;
        const uint32_t subj = a.n_subj - 1 - static_cast<uint32_t>(t);
        const uint64_t o0 = a.off[subj];
        wf.slen = static_cast<int32_t>(a.off[subj + 1] - o0);
        wf.n_init = 0;
        residues += static_cast<unsigned long long>(wf.slen);
        if (static_cast<uint32_t>(wf.slen) <= a.stage_bytes) {
            // stage the subject: 16-byte aligned vectors covering it (the
            // database is padded, so the last vector stays in bounds)
            const uint32_t lead = static_cast<uint32_t>(o0 & 15u);
            const uint4 *src = reinterpret_cast<const uint4 *>(a.res + (o0 - lead));
            const uint32_t nvec = (lead + static_cast<uint32_t>(wf.slen) + 15u) >> 4;
            for (uint32_t i = lane; i < nvec; i += 32) reinterpret_cast<uint4 *>(stage)[i] = __ldg(src + i);
            __syncwarp();
            wf.sub = stage + lead;
        } else {
            wf.sub = a.res + o0;
        }
        const int32_t nwords = wf.slen - (kWordSize - 1);
        // chunks of 128 word positions, four consecutive positions per lane
        for (int32_t cb = 0; cb < nwords; cb += 4 * 32) {
            const int32_t p0 = cb + 4 * lane;
            int32_t r[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) r[j] = wf.sub[min(p0 + j, wf.slen - 1)];
            uint32_t cs[4], cnt[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int w = r[j] * 784 + r[j + 1] * 28 + r[j + 2];
                const bool present = p0 + j < nwords && ((presence[w >> 5] >> (w & 31)) & 1u);
                const uint32_t pk = present ? __ldg(a.cell_pack + w) : 0u;
                cs[j] = pk >> 8;
                cnt[j] = pk & 0xffu;
                if (cnt[j] == 0xffu) cnt[j] = __ldg(a.cell_start + w + 1) - cs[j];
            }
            const uint32_t mine_total = cnt[0] + cnt[1] + cnt[2] + cnt[3];
            uint32_t incl = mine_total;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += x;
            }
            const uint32_t total = __shfl_sync(kFull, incl, 31);
            if (total == 0) continue;
            word_hits += total;
            const uint32_t e0 = incl - mine_total, e1 = e0 + cnt[0], e2 = e1 + cnt[1], e3 = e2 + cnt[2];
            for (uint32_t kb = 0; kb < total; kb += 32) {
                const uint32_t k = kb + lane;
                // owner lane: the last lane whose first hit index is <= k
                int lo = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const uint32_t ev = __shfl_sync(kFull, e0, lo + step);
                    if (ev <= k) lo += step;
                }
                // owner position: the last of its four whose first hit is <= k
                const uint32_t E0 = __shfl_sync(kFull, e0, lo), E1 = __shfl_sync(kFull, e1, lo);
                const uint32_t E2 = __shfl_sync(kFull, e2, lo), E3 = __shfl_sync(kFull, e3, lo);
                const uint32_t C0 = __shfl_sync(kFull, cs[0], lo), C1 = __shfl_sync(kFull, cs[1], lo);
                const uint32_t C2 = __shfl_sync(kFull, cs[2], lo), C3 = __shfl_sync(kFull, cs[3], lo);
                const int j = (k >= E1) + (k >= E2) + (k >= E3);
                const uint32_t Ej = j == 0 ? E0 : j == 1 ? E1 : j == 2 ? E2 : E3;
                const uint32_t Cj = j == 0 ? C0 : j == 1 ? C1 : j == 2 ? C2 : C3;
                const bool hv = k < total;
                const int32_t qo = hv ? static_cast<int32_t>(__ldg(a.cell_off + Cj + (k - Ej))) : 0;
                process_batch(wf, a, hv, cb + 4 * lo + j, qo);
                if (wf.n_seed >= 32 || wf.n_defer > kDeferCap - 32) flush(wf, a, mat);
            }
        }
        flush(wf, a, mat);

        // publish this subject's init hits as one contiguous block
        if (wf.n_init > 0) {
            if (wf.n_init > a.scratch_cap) {
                if (lane == 0) {
                    atomicAdd(&a.cnt->overflow_subjects, 1u);
                    atomicMax(&a.cnt->max_init_needed, wf.n_init);
                }
            } else {
                unsigned long long first = 0, wi = 0;
                if (lane == 0) {
                    first = atomicAdd(&a.cnt->init_count, static_cast<unsigned long long>(wf.n_init));
                    wi = atomicAdd(&a.cnt->work_count, 1ull);
                }
                first = __shfl_sync(kFull, first, 0);
                wi = __shfl_sync(kFull, wi, 0);
                if (first + wf.n_init > a.init_cap || wi >= a.work_cap) {
                    if (lane == 0)
                        atomicOr(&a.cnt->flags, first + wf.n_init > a.init_cap ? kFlagInitArrayFull : kFlagWorkArrayFull);
                } else {
                    for (uint32_t i = lane; i < wf.n_init; i += 32) a.init_out[first + i] = wf.scratch[i];
                    if (lane == 0) {
                        WorkItem w;
                        w.subject = subj;
                        w.n_init = wf.n_init;
                        w.first = first;
                        a.work[wi] = w;
                    }
                }
            }
        }
        wf.base += static_cast<uint32_t>(wf.slen + a.window);
        __syncwarp();
        if (wf.base > kBaseReset) {
            for (uint32_t i = lane; i < a.diag_entries; i += 32) wf.diag[i] = 0;
            wf.base = 0;
            __syncwarp();
        }
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->word_hits, word_hits);
        atomicAdd(&a.cnt->residues, residues);
        atomicAdd(&a.cnt->extensions, wf.extensions);
    }
}

}  // namespace

ScanLayout scan_layout(int32_t qlen, int32_t window, uint32_t stage_bytes, size_t smem_budget) {
    ScanLayout l{};
    l.diag_entries = static_cast<uint32_t>(qlen + window + 3) & ~3u;  // >= qlen + window
    l.diag_magic = static_cast<uint32_t>((1ull << 32) / l.diag_entries + 1);
    l.diag_bytes = l.diag_entries * 4u;
    l.stage_bytes = stage_bytes;
    l.query_smem_bytes = qlen <= kQuerySmemMax ? (static_cast<uint32_t>(qlen) + 15u) & ~15u : 0u;
    l.warp_smem_bytes = l.diag_bytes + 2 * kDeferCap * sizeof(uint2) + kSeedCap * sizeof(int4) +
                        ((stage_bytes + 32u + 15u) & ~15u);
    const size_t fixed = kScanMatBytes + kScanPresenceBytes + l.query_smem_bytes;
    int w = kScanMaxWarpsPerBlock;
    while (w > 1 && fixed + static_cast<size_t>(w) * l.warp_smem_bytes > smem_budget) --w;
    l.warps_per_block = w;
    l.smem_bytes = fixed + static_cast<size_t>(w) * l.warp_smem_bytes;
    return l;
}

cudaError_t launch_scan(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    scan_kernel<<<n_blocks, warps_per_block * 32, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t scan_occupancy(int warps_per_block, size_t smem, int *blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, scan_kernel,
                                                         warps_per_block * 32, smem);
}

}  // namespace blaze
