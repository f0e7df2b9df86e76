// scan.cu -- word finder, two-hit seeding and ungapped X-drop extension of
// the BLASTP preliminary search on GB300 (sm_103a). Integer work only.
//
// One warp per subject; persistent warps pull subjects, longest first, from a
// device cursor (batched: blocks pull (query, subject range) tiles, their
// warps the tile's subjects). Per block in shared memory: the BLOSUM62 matrix
// (int8), the query's word-presence bitset and, for queries up to
// kQuerySmemMax, the query residues. Per warp: the diagonal table, the deferred-hit and seed
// queues and a staging buffer that holds the whole subject when it fits, so
// the word scan and the extensions read shared memory instead of making
// dependent global loads.
//
// Reference counterpart: gpuBLAZE_full (BLAZE_gpu/gpuBLAZE.cu:885-1252), which
// is a filter; this kernel produces the exact ungapped HSPs of the
// sequential algorithm.
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <set>
#include <utility>

#include "common.cuh"

namespace blaze {
namespace {

__device__ const int8_t g_blosum8[kAlphabet * kAlphabet] = {
#include "blosum62_i8.inc"
};

constexpr unsigned kFull = 0xffffffffu;
constexpr int kCoopSeeds = 4;  // flushes with at most this many seeds extend warp-cooperatively
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
// Shared-memory layout (byte offsets into the dynamic array). Every table is
// reached through a 32-bit offset into `smem` itself, so all of them compile
// to shared-space accesses.

constexpr uint32_t kMatOff = 0;
constexpr uint32_t kPresOff = kScanMatBytes;
constexpr uint32_t kQueryOff = kScanMatBytes + kScanPresenceBytes;

extern __shared__ __align__(16) unsigned char smem[];

__device__ __forceinline__ uint32_t lds32(uint32_t off) { return reinterpret_cast<const uint32_t *>(smem)[off >> 2]; }
__device__ __forceinline__ void sts32(uint32_t off, uint32_t v) { reinterpret_cast<uint32_t *>(smem)[off >> 2] = v; }
__device__ __forceinline__ int32_t score_of(uint32_t qa, uint32_t sb) {
    return static_cast<int32_t>(reinterpret_cast<const int8_t *>(smem)[kMatOff + qa * kAlphabet + sb]);
}

// ------------------------------------------------------------------------
// Subject staging by the bulk-copy (TMA) engine: one elected lane arms the
// warp's mbarrier with the byte count and issues cp.async.bulk
// global -> shared; the warp waits on the barrier's phase. A warp stages one
// subject at a time, just before scanning it, in one stage buffer. Waits are
// bounded: a copy that never lands sets kFlagBadState.

constexpr uint32_t kBulkSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_base() { return static_cast<uint32_t>(__cvta_generic_to_shared(smem)); }

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0u;
}

// Lane 0 of the calling warp: copies `bytes` (a multiple of 16) from 16-byte
// aligned global `src` to shared offset `dst` and completes the barrier.
__device__ __forceinline__ void bulk_stage(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    const uint32_t d = smem_base() + dst, b = smem_base() + bar;
    // earlier generic reads of this buffer come before the async overwrite
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(d), "l"(src), "r"(bytes), "r"(b)
                 : "memory");
}

// The subject: staged in shared memory, or read from global memory when it is
// longer than the staging buffer.
template <bool STAGED>
struct Subject {
    uint32_t off;        // shared offset of residue 0 (staged)
    const uint8_t *ptr;  // global address of residue 0 (not staged)
    int32_t len;
    __device__ __forceinline__ uint32_t at(int32_t i) const {
        if (STAGED) return smem[off + i];
        return __ldg(ptr + i);
    }
};

// The query: in shared memory for queries up to kQuerySmemMax, else global.
template <bool QSMEM>
struct Query {
    const uint8_t *ptr;
    int32_t len;
    __device__ __forceinline__ uint32_t at(int32_t i) const {
        if (QSMEM) return smem[kQueryOff + i];
        return __ldg(ptr + i);
    }
};

// ------------------------------------------------------------------------
// Ungapped extension (scalar, one lane per seed), same walks as the oracle:
// left from the end of the best word prefix, right only when the left walk
// reached the first hit (BLAZE_gpu/gpuBLAZE.cu:1096-1152 is the warp form).

template <bool QS, bool ST>
__device__ __forceinline__ int32_t extend_left(const Query<QS> &q, const Subject<ST> &s, int32_t q_off,
                                               int32_t s_off, int32_t xdrop, int32_t *length) {
    const int32_t n = min(s_off, q_off);
    int32_t best_k = -1, score = 0, maxscore = 0;
    for (int32_t k = 0; k <= n; ++k) {
        score += score_of(q.at(q_off - k), s.at(s_off - k));
        if (score > maxscore) {
            maxscore = score;
            best_k = k;
        }
        if (maxscore - score >= xdrop) break;
    }
    *length = best_k + 1;
    return maxscore;
}

template <bool QS, bool ST>
__device__ __forceinline__ int32_t extend_right(const Query<QS> &q, const Subject<ST> &s, int32_t q_off,
                                                int32_t s_off, int32_t xdrop, int32_t maxscore,
                                                int32_t *length, int32_t *s_last_off) {
    const int32_t n = min(s.len - s_off, q.len - q_off);
    int32_t best_i = -1, score = maxscore, i;
    for (i = 0; i < n; ++i) {
        score += score_of(q.at(q_off + i), s.at(s_off + i));
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

template <bool QS, bool ST>
__device__ __forceinline__ int32_t extend_two_hit(const Query<QS> &q, const Subject<ST> &s,
                                                  int32_t s_left_off, int32_t s_off, int32_t q_off,
                                                  int32_t xdrop, int32_t *hsp_q, int32_t *hsp_s,
                                                  int32_t *hsp_len, int32_t *right_extend,
                                                  int32_t *s_last_off) {
    int32_t score = 0, left_score = 0, right_d = 0, left_d = 0, right_score = 0;
#pragma unroll
    for (int32_t i = 0; i < kWordSize; ++i) {
        score += score_of(q.at(q_off + i), s.at(s_off + i));
        if (score > left_score) {
            left_score = score;
            right_d = i + 1;
        }
    }
    const int32_t q_right = q_off + right_d, s_right = s_off + right_d;
    left_score = extend_left(q, s, q_right - 1, s_right - 1, xdrop, &left_d);
    right_d = 0;
    *right_extend = 0;
    *s_last_off = s_right;
    if (left_d >= s_right - s_left_off) {
        *right_extend = 1;
        right_score = extend_right(q, s, q_right, s_right, xdrop, left_score, &right_d, s_last_off);
    }
    *hsp_q = q_right - left_d;
    *hsp_s = s_right - left_d;
    *hsp_len = left_d + right_d;
    return max(left_score, right_score);
}

// ------------------------------------------------------------------------
// Warp-cooperative form of extend_two_hit for one seed: the 32 lanes take 32
// consecutive positions of a walk per step. The running score is a prefix sum
// and the running best a prefix maximum (carried between steps); the walk
// stops at the first position whose stop test holds, and the best is the
// first position reaching the final maximum -- exactly the positions and
// scores of the sequential walk. Every lane returns the same values.

// One X-drop walk of up to n positions; score and best start at `start`.
// t(k) gives the score of the k-th position. Returns the best score; *best_k
// is its position (-1 when never above start), *end the position the walk
// stopped at (n when it ran out). right: also stop when the score drops to 0.
template <bool RIGHT, typename F>
__device__ __forceinline__ int32_t walk_warp(F t, int32_t n, int32_t start, int32_t xdrop, int32_t *best_k,
                                             int32_t *end) {
    const int lane = threadIdx.x & 31;
    int32_t carry = start, cmax = start, bk = -1, stop_at = n;
    for (int32_t base = 0; base < n; base += 32) {
        const int32_t k = base + lane;
        const bool valid = k < n;
        int32_t S = valid ? t(k) : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t x = __shfl_up_sync(kFull, S, o);
            if (lane >= o) S += x;
        }
        S += carry;
        int32_t P = S;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t x = __shfl_up_sync(kFull, P, o);
            if (lane >= o) P = max(P, x);
        }
        P = max(P, cmax);
        const bool stop = valid && ((RIGHT && S <= 0) || P - S >= xdrop);
        const unsigned sm = __ballot_sync(kFull, stop);
        const int last = sm ? __ffs(sm) - 1 : min(31, n - 1 - base);
        const int32_t m = __shfl_sync(kFull, P, last);
        if (m > cmax) {
            const unsigned hm = __ballot_sync(kFull, valid && lane <= last && S == m);
            bk = base + __ffs(hm) - 1;
            cmax = m;
        }
        carry = __shfl_sync(kFull, S, last);
        if (sm) {
            stop_at = base + last;
            break;
        }
    }
    *best_k = bk;
    *end = stop_at;
    return cmax;
}

template <bool QS, bool ST>
__device__ __forceinline__ int32_t extend_two_hit_warp(const Query<QS> &q, const Subject<ST> &s,
                                                       int32_t s_left_off, int32_t s_off, int32_t q_off,
                                                       int32_t xdrop, int32_t *hsp_q, int32_t *hsp_s,
                                                       int32_t *hsp_len, int32_t *right_extend,
                                                       int32_t *s_last_off) {
    int32_t score = 0, left_score = 0, right_d = 0;
#pragma unroll
    for (int32_t i = 0; i < kWordSize; ++i) {
        score += score_of(q.at(q_off + i), s.at(s_off + i));
        if (score > left_score) {
            left_score = score;
            right_d = i + 1;
        }
    }
    const int32_t q_right = q_off + right_d, s_right = s_off + right_d;
    // left: positions k = 0 .. min(s_right, q_right) - 1 backwards from the
    // residue pair before (q_right, s_right)
    int32_t bk, end;
    left_score = walk_warp<false>(
        [&](int32_t k) { return score_of(q.at(q_right - 1 - k), s.at(s_right - 1 - k)); },
        min(s_right, q_right), 0, xdrop, &bk, &end);
    const int32_t left_d = bk + 1;
    int32_t right_score = 0, rd = 0;
    *right_extend = 0;
    *s_last_off = s_right;
    if (left_d >= s_right - s_left_off) {
        *right_extend = 1;
        int32_t bi, iend;
        right_score = walk_warp<true>(
            [&](int32_t i) { return score_of(q.at(q_right + i), s.at(s_right + i)); },
            min(s.len - s_right, q.len - q_right), left_score, xdrop, &bi, &iend);
        rd = bi + 1;
        *s_last_off = s_right + iend;
    }
    *hsp_q = q_right - left_d;
    *hsp_s = s_right - left_d;
    *hsp_len = left_d + rd;
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

struct Finder {
    uint32_t diag, defer, seeds;  // shared offsets
    uint32_t bars;                // the two stage buffers' mbarriers
    uint32_t phase;               // bit b: parity the next wait on buffer b expects
    int n_defer, n_seed, sel;
    uint32_t base;
    uint32_t n_init;
    InitHit *scratch;
    unsigned long long extensions;
};

// Per-query parameters of the word finder (one query, or the query of the
// current tile in a batch).
struct Ctx {
    const uint8_t *q;
    int32_t qlen;
    const uint32_t *cell_start, *cell_pack, *presence;
    const uint16_t *cell_off;
    uint32_t diag_entries, diag_magic;
    int32_t window, xdrop, cutoff;
};

__device__ __forceinline__ void put_defer(const Finder &f, int buf, int i, int32_t s, int32_t q) {
    reinterpret_cast<uint2 *>(smem)[(f.defer >> 3) + buf * kDeferCap + i] =
        make_uint2(static_cast<uint32_t>(s), static_cast<uint32_t>(q));
}
__device__ __forceinline__ uint2 get_defer(const Finder &f, int buf, int i) {
    return reinterpret_cast<const uint2 *>(smem)[(f.defer >> 3) + buf * kDeferCap + i];
}
__device__ __forceinline__ void put_seed(const Finder &f, int i, int4 v) {
    reinterpret_cast<int4 *>(smem)[(f.seeds >> 4) + i] = v;
}
__device__ __forceinline__ int4 get_seed(const Finder &f, int i) {
    return reinterpret_cast<const int4 *>(smem)[(f.seeds >> 4) + i];
}

// Runs up to 32 hits (one per lane, lanes in hit order) through the two-hit
// logic. Hits on the same diagonal are taken in lane order; a hit whose
// diagonal waits on an extension is appended to the deferred list.
__device__ __forceinline__ void process_batch(Finder &f, const Ctx &c, bool valid, int32_t s,
                                              int32_t q) {
    if (__ballot_sync(kFull, valid) == 0) return;
    const uint32_t d = fast_mod(static_cast<uint32_t>(s - q + c.qlen), c.diag_entries, c.diag_magic);
    const uint32_t doff = f.diag + 4u * d;
    const unsigned lt = lanemask_lt();
    const unsigned peers = __match_any_sync(kFull, valid ? d : 0xffffffffu);
    const unsigned rank = valid ? __popc(peers & lt) : 0u;
    const unsigned max_rank = __reduce_max_sync(kFull, rank);
    const uint32_t here = static_cast<uint32_t>(s + c.window) + f.base;  // s, biased
    for (unsigned r = 0; r <= max_rank; ++r) {
        const bool mine = valid && rank == r;
        const uint32_t e = mine ? lds32(doff) : 0u;
        const bool pend = (e & kPendBit) != 0u;
        const bool flag = (e & kFlagBit) != 0u;
        const int32_t last = static_cast<int32_t>(e & kValMask) - c.window - static_cast<int32_t>(f.base);
        const int32_t diff = s - last;
        // flag set: hits inside the last extension are skipped, the first one
        // past it starts over; otherwise a hit far from the last one starts
        // over, one at distance [wordsize, window) triggers an extension, and
        // an overlapping one is ignored
        const bool defer = mine && pend;
        const bool seed = mine && !pend && !flag && diff >= kWordSize && diff < c.window;
        const bool set = mine && !pend && (flag ? s >= last : diff >= c.window);
        if (set) sts32(doff, here);
        const unsigned dm = __ballot_sync(kFull, defer);
        const unsigned sm = __ballot_sync(kFull, seed);
        if ((dm | sm) != 0u) {
            if (defer) put_defer(f, f.sel, f.n_defer + __popc(dm & lt), s, q);
            if (seed) {
                const int slot = f.n_seed + __popc(sm & lt);
                put_seed(f, slot, make_int4(q, s, last + kWordSize, static_cast<int32_t>(d)));
                sts32(doff, kPendBit | static_cast<uint32_t>(slot));
            }
            f.n_defer += __popc(dm);
            f.n_seed += __popc(sm);
        }
        __syncwarp();
    }
}

// Extends every queued seed (one lane each), settles their diagonals, keeps
// those reaching the ungapped cutoff, then replays the deferred hits; repeats
// until no seed and no deferred hit is left. Each replay is shorter than the
// list it replays whenever it queues a seed, so the loop ends.
template <bool QS, bool ST>
__device__ void flush(Finder &f, const ScanArgs &a, const Ctx &c, const Query<QS> &q,
                      const Subject<ST> &sub) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    while (f.n_seed > 0 || f.n_defer > 0) {
        // few seeds: one at a time with the whole warp on each walk
        for (int i = 0; f.n_seed <= kCoopSeeds && i < f.n_seed; ++i) {
            const int4 sd = get_seed(f, i);
            int32_t hq, hs, hl, rext, slast;
            const int32_t score =
                extend_two_hit_warp(q, sub, sd.z, sd.y, sd.x, c.xdrop, &hq, &hs, &hl, &rext, &slast);
            if (lane == 0) {
                sts32(f.diag + 4u * static_cast<uint32_t>(sd.w),
                      rext ? (kFlagBit | (static_cast<uint32_t>(slast - (kWordSize - 1) + c.window) + f.base))
                           : (static_cast<uint32_t>(sd.y + c.window) + f.base));
                if (score >= c.cutoff && f.n_init < a.scratch_cap) {
                    InitHit h;
                    h.q_start = hq;
                    h.s_start = hs;
                    h.len = hl;
                    h.score = score;
                    h.q_trig = sd.x;
                    h.s_trig = sd.y;
                    f.scratch[f.n_init] = h;
                }
            }
            if (score >= c.cutoff) ++f.n_init;
        }
        // many: one lane per seed
        for (int c0 = 0; f.n_seed > kCoopSeeds && c0 < f.n_seed; c0 += 32) {
            const int i = c0 + lane;
            bool pass = false;
            int32_t hq = 0, hs = 0, hl = 0, score = 0;
            int4 sd = make_int4(0, 0, 0, 0);
            if (i < f.n_seed) {
                sd = get_seed(f, i);
                int32_t rext, slast;
                score = extend_two_hit(q, sub, sd.z, sd.y, sd.x, c.xdrop, &hq, &hs, &hl, &rext, &slast);
                sts32(f.diag + 4u * static_cast<uint32_t>(sd.w),
                      rext ? (kFlagBit | (static_cast<uint32_t>(slast - (kWordSize - 1) + c.window) + f.base))
                           : (static_cast<uint32_t>(sd.y + c.window) + f.base));
                pass = score >= c.cutoff;
            }
            const unsigned pm = __ballot_sync(kFull, pass);
            if (pass) {
                const uint32_t pos = f.n_init + __popc(pm & lt);
                if (pos < a.scratch_cap) {
                    InitHit h;
                    h.q_start = hq;
                    h.s_start = hs;
                    h.len = hl;
                    h.score = score;
                    h.q_trig = sd.x;
                    h.s_trig = sd.y;
                    f.scratch[pos] = h;
                }
            }
            f.n_init += __popc(pm);
        }
        f.extensions += static_cast<unsigned long long>(f.n_seed);
        f.n_seed = 0;
        __syncwarp();
        if (f.n_defer > 0) {
            const int old = f.sel, n_old = f.n_defer;
            f.sel ^= 1;
            f.n_defer = 0;
            for (int c0 = 0; c0 < n_old; c0 += 32) {
                const int i = c0 + lane;
                const bool v = i < n_old;
                const uint2 h = v ? get_defer(f, old, i) : make_uint2(0u, 0u);
                process_batch(f, c, v, static_cast<int32_t>(h.x), static_cast<int32_t>(h.y));
            }
        }
    }
}

// Word scan of one subject: chunks of 128 positions, four consecutive
// positions per lane; one warp prefix sum per chunk lays the hits out in
// (subject offset, query offset) order, and lanes take them 32 at a time.
template <bool QS, bool ST, bool PSMEM>
__device__ __forceinline__ unsigned long long scan_subject(Finder &f, const ScanArgs &a, const Ctx &c,
                                                           const Query<QS> &q, const Subject<ST> &sub) {
    const int lane = threadIdx.x & 31;
    unsigned long long word_hits = 0;
    const int32_t nwords = sub.len - (kWordSize - 1);
    for (int32_t cb = 0; cb < nwords; cb += 4 * 32) {
        const int32_t p0 = cb + 4 * lane;
        uint32_t r[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) r[j] = sub.at(min(p0 + j, sub.len - 1));
        uint32_t cs[4], cnt[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t w = r[j] * 784u + r[j + 1] * 28u + r[j + 2];
            const uint32_t pw = PSMEM ? lds32(kPresOff + 4u * (w >> 5)) : __ldg(c.presence + (w >> 5));
            const bool present = p0 + j < nwords && ((pw >> (w & 31u)) & 1u);
            const uint32_t pk = present ? __ldg(c.cell_pack + w) : 0u;
            cs[j] = pk >> 8;
            cnt[j] = pk & 0xffu;
            if (cnt[j] == 0xffu) cnt[j] = __ldg(c.cell_start + w + 1) - cs[j];
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
            const int32_t qo = hv ? static_cast<int32_t>(__ldg(c.cell_off + Cj + (k - Ej))) : 0;
            process_batch(f, c, hv, cb + 4 * lo + j, qo);
            if (f.n_seed >= 32 || f.n_defer > kDeferCap - 32) flush(f, a, c, q, sub);
        }
    }
    flush(f, a, c, q, sub);
    return word_hits;
}

constexpr uint32_t kNoStage = 0xffffffffu;

__device__ __forceinline__ uint32_t stage_region(const ScanArgs &a) { return (a.stage_bytes + 32u + 15u) & ~15u; }

// Issues the bulk copy of subject `subj` into stage buffer `buf` when it is
// long enough to have a word and fits; returns whether it did.
__device__ __forceinline__ bool stage_issue(const Finder &f, const ScanArgs &a, uint32_t stage, int buf,
                                            uint32_t subj) {
    const uint64_t o0 = a.off[subj];
    const uint64_t slen = a.off[subj + 1] - o0;
    if (slen < static_cast<uint64_t>(kWordSize) || slen > a.stage_bytes) return false;
    const uint32_t lead = static_cast<uint32_t>(o0 & 15u);
    const uint32_t bytes = (lead + static_cast<uint32_t>(slen) + 15u) & ~15u;  // the database is padded
    if ((threadIdx.x & 31) == 0)
        bulk_stage(stage + static_cast<uint32_t>(buf) * stage_region(a), a.res + (o0 - lead), bytes,
                   f.bars + 8u * static_cast<uint32_t>(buf));
    return true;
}

// Waits for buffer `buf`'s copy; false (with kFlagBadState set) if it never
// completes within the spin limit.
__device__ __forceinline__ bool stage_wait(Finder &f, const ScanArgs &a, int buf) {
    const uint32_t bar = smem_base() + f.bars + 8u * static_cast<uint32_t>(buf);
    const uint32_t parity = (f.phase >> buf) & 1u;
    for (uint32_t i = 0; i < kBulkSpinLimit; ++i) {
        if (mbar_try_wait(bar, parity)) {
            f.phase ^= 1u << buf;
            return true;
        }
    }
    if ((threadIdx.x & 31) == 0) atomicOr(&a.cnt->flags, kFlagBadState);
    return false;
}

// One subject for the query of `c` (staged at shared offset `staged` by a
// bulk copy, or read from global memory): find its init hits and publish
// them as one contiguous block with a work item.
template <bool QS, bool PSMEM>
__device__ __forceinline__ void process_subject(Finder &f, const ScanArgs &a, const Ctx &c, const Query<QS> &q,
                                                uint32_t subj, uint32_t query_index, uint32_t staged,
                                                unsigned long long &word_hits, unsigned long long &residues) {
    const int lane = threadIdx.x & 31;
    const uint64_t o0 = a.off[subj];
    const int32_t slen = static_cast<int32_t>(a.off[subj + 1] - o0);
    f.n_init = 0;
    residues += static_cast<unsigned long long>(slen);
    if (staged != kNoStage) {
        Subject<true> sub;
        sub.off = staged + static_cast<uint32_t>(o0 & 15u);
        sub.ptr = nullptr;
        sub.len = slen;
        word_hits += scan_subject<QS, true, PSMEM>(f, a, c, q, sub);
    } else {
        Subject<false> sub;
        sub.off = 0;
        sub.ptr = a.res + o0;
        sub.len = slen;
        word_hits += scan_subject<QS, false, PSMEM>(f, a, c, q, sub);
    }

    // publish this subject's init hits as one contiguous block
    if (f.n_init > 0) {
        if (f.n_init > a.scratch_cap) {
            if (lane == 0) {
                atomicAdd(&a.cnt->overflow_subjects, 1u);
                atomicMax(&a.cnt->max_init_needed, f.n_init);
            }
        } else {
            unsigned long long first = 0, wi = 0;
            if (lane == 0) {
                first = atomicAdd(&a.cnt->init_count, static_cast<unsigned long long>(f.n_init));
                wi = atomicAdd(&a.cnt->work_count, 1ull);
            }
            first = __shfl_sync(kFull, first, 0);
            wi = __shfl_sync(kFull, wi, 0);
            if (first + f.n_init > a.init_cap || wi >= a.work_cap) {
                if (lane == 0) {
                    atomicOr(&a.cnt->flags, first + f.n_init > a.init_cap ? kFlagInitArrayFull : kFlagWorkArrayFull);
                    if (wi < a.work_cap) {  // a counted slot always holds an item: an empty one
                        WorkItem w;
                        w.subject = subj;
                        w.n_init = 0;
                        w.first = 0;
                        a.work[wi] = w;
                        if (a.work_query) a.work_query[wi] = query_index;
                    }
                }
            } else {
                for (uint32_t i = lane; i < f.n_init; i += 32) a.init_out[first + i] = f.scratch[i];
                if (lane == 0) {
                    WorkItem w;
                    w.subject = subj;
                    w.n_init = f.n_init;
                    w.first = first;
                    a.work[wi] = w;
                    if (a.work_query) a.work_query[wi] = query_index;
                }
            }
        }
    }
    f.base += static_cast<uint32_t>(slen + c.window);
    __syncwarp();
    if (f.base > kBaseReset) {
        for (uint32_t i = lane; i < c.diag_entries; i += 32) sts32(f.diag + 4u * i, 0u);
        f.base = 0;
        __syncwarp();
    }
}

__device__ __forceinline__ Finder make_finder(const ScanArgs &a, uint32_t qbytes, uint32_t &stage) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t mine = kQueryOff + qbytes + static_cast<uint32_t>(warp) * a.warp_smem_bytes;
    Finder f;
    f.diag = mine;
    f.defer = mine + a.diag_bytes;
    f.seeds = f.defer + 2u * kDeferCap * sizeof(uint2);
    f.bars = f.seeds + kSeedCap * sizeof(int4);  // two 8-byte mbarriers, 16 bytes
    stage = f.bars + 16u;                         // two stage buffers of stage_region bytes
    f.phase = 0u;
    if (lane == 0) {
        mbar_init(smem_base() + f.bars);
        mbar_init(smem_base() + f.bars + 8u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    f.n_defer = f.n_seed = f.sel = 0;
    f.base = 0;
    f.extensions = 0;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    f.scratch = a.scratch + gwarp * a.scratch_cap;
    for (uint32_t i = lane; i < a.diag_entries_max; i += 32) sts32(f.diag + 4u * i, 0u);
    return f;
}

__device__ __forceinline__ void finish_counters(const ScanArgs &a, const Finder &f, unsigned long long word_hits,
                                                unsigned long long residues) {
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&a.cnt->word_hits, word_hits);
        atomicAdd(&a.cnt->residues, residues);
        atomicAdd(&a.cnt->extensions, f.extensions);
    }
}

// One query against the whole database: the query's presence bitset (and
// the query itself when short enough) live in shared memory; warps pull
// subjects longest first.
template <bool QS>
__global__ void __launch_bounds__(kScanMaxWarpsPerBlock * 32, 1)
scan_kernel(const ScanArgs a) {
    const int lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x)
        reinterpret_cast<int8_t *>(smem)[kMatOff + i] = g_blosum8[i];
    for (int i = threadIdx.x; i < kPresenceWords; i += blockDim.x) sts32(kPresOff + 4u * i, a.presence[i]);
    if (QS)
        for (int i = threadIdx.x; i < a.qlen; i += blockDim.x) smem[kQueryOff + i] = a.q[i];
    uint32_t stage = 0;
    Finder f = make_finder(a, a.query_smem_bytes, stage);
    __syncthreads();
    Ctx c;
    c.q = a.q;
    c.qlen = a.qlen;
    c.cell_start = a.cell_start;
    c.cell_pack = a.cell_pack;
    c.presence = a.presence;
    c.cell_off = a.cell_off;
    c.diag_entries = a.diag_entries;
    c.diag_magic = a.diag_magic;
    c.window = a.window;
    c.xdrop = a.xdrop;
    c.cutoff = a.cutoff;
    Query<QS> q;
    q.ptr = a.q;
    q.len = a.qlen;
    unsigned long long word_hits = 0, residues = 0;
    const unsigned long long count = a.n_subj;
    auto next = [&]() {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(a.cursor, 1ull);
        return __shfl_sync(kFull, t, 0);
    };
    // subjects longest first, each staged by a bulk copy when it fits
    for (unsigned long long t = next(); t < count; t = next()) {
        const uint32_t subj = a.n_subj - 1 - static_cast<uint32_t>(t);
        const bool staged = stage_issue(f, a, stage, 0, subj);
        if (staged && !stage_wait(f, a, 0)) return;
        process_subject<QS, true>(f, a, c, q, subj, a.query_index, staged ? stage : kNoStage, word_hits,
                                  residues);
    }
    finish_counters(a, f, word_hits, residues);
}

// Many queries against the database: blocks pull (query, subject range)
// tiles; tile t covers query t mod n_queries and the (t / n_queries)-th
// range counted from the longest subjects down, so every query's long
// subjects come first and queries interleave. Ranges hold about equal
// residues (host-computed bounds, sized for a whole block). A block stages
// its tile's query tables in shared memory -- the word-presence bitset and,
// up to kQuerySmemMax residues, the query -- and lays its warps' regions out
// for that query: each warp's diagonal table takes the query's length plus
// the window, so as many warps as fit (at most the block's) take the range's
// subjects, longest first, from a shared cursor; the others sit the tile out.
// The block restages only after every warp has left the tile. Shared memory:
// matrix, presence bitset, query, one pair of mbarriers per warp, then the
// warps' regions (diagonal table, deferred hits, seeds, stage buffer).
template <bool QS>
__global__ void __launch_bounds__(kScanMaxWarpsPerBlock * 32, 1)
scan_batch_kernel(const ScanArgs a) {
    __shared__ unsigned long long s_tile;
    __shared__ uint32_t s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n_warps = blockDim.x >> 5;
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x)
        reinterpret_cast<int8_t *>(smem)[kMatOff + i] = g_blosum8[i];
    const uint32_t bars = kQueryOff + a.query_smem_bytes;  // 16-byte aligned
    const uint32_t regions = bars + 16u * n_warps;
    Finder f;
    f.bars = bars + 16u * static_cast<uint32_t>(warp);
    f.phase = 0u;
    f.n_defer = f.n_seed = f.sel = 0;
    f.base = 0;
    f.extensions = 0;
    f.n_init = 0;
    f.scratch = a.scratch + ((static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) *
                                a.scratch_cap;
    if (lane == 0) {
        mbar_init(smem_base() + f.bars);
        mbar_init(smem_base() + f.bars + 8u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const unsigned long long n_tiles = static_cast<unsigned long long>(a.n_ranges) * a.n_queries;
    const uint32_t fixed_warp_bytes = 2u * kDeferCap * sizeof(uint2) + kSeedCap * sizeof(int4) + stage_region(a);
    unsigned long long word_hits = 0, residues = 0;
    bool staging = true;  // false after a bulk copy that never landed (kFlagBadState is set)
    for (;;) {
        if (threadIdx.x == 0) {
            s_tile = atomicAdd(a.cursor, 1ull);
            s_next = 0u;
        }
        __syncthreads();  // also orders the previous tile's last table reads before the restage
        const unsigned long long t = s_tile;
        if (t >= n_tiles) break;
        const uint32_t qi = static_cast<uint32_t>(t % a.n_queries);
        const uint32_t range = static_cast<uint32_t>(t / a.n_queries);
        const BatchQuery bq = a.queries[qi];
        for (int i = threadIdx.x; i < kPresenceWords; i += blockDim.x) sts32(kPresOff + 4u * i, bq.presence[i]);
        if (QS)
            for (int i = threadIdx.x; i < bq.qlen; i += blockDim.x) smem[kQueryOff + i] = bq.q[i];
        __syncthreads();
        const uint32_t diag_bytes = (4u * bq.diag_entries + 15u) & ~15u;
        const uint32_t warp_bytes = diag_bytes + fixed_warp_bytes;
        const uint32_t active = min(n_warps, (a.smem_bytes - regions) / warp_bytes);  // >= 1 (host)
        if (static_cast<uint32_t>(warp) < active) {
            f.diag = regions + static_cast<uint32_t>(warp) * warp_bytes;
            f.defer = f.diag + diag_bytes;
            f.seeds = f.defer + 2u * kDeferCap * sizeof(uint2);
            const uint32_t stage = f.seeds + kSeedCap * sizeof(int4);
            for (uint32_t i = lane; i < bq.diag_entries; i += 32) sts32(f.diag + 4u * i, 0u);
            f.base = 0;
            __syncwarp();
            Ctx c;
            c.q = bq.q;
            c.qlen = bq.qlen;
            c.cell_start = bq.cell_start;
            c.cell_pack = bq.cell_pack;
            c.presence = bq.presence;
            c.cell_off = bq.cell_off;
            c.diag_entries = bq.diag_entries;
            c.diag_magic = bq.diag_magic;
            c.window = a.window;
            c.xdrop = a.xdrop;
            c.cutoff = bq.ungapped_cutoff;
            Query<QS> q;
            q.ptr = bq.q;
            q.len = bq.qlen;
            const uint32_t hi = a.tile_bounds[range], lo = a.tile_bounds[range + 1];
            for (;;) {
                uint32_t k = 0;
                if (lane == 0) k = atomicAdd(&s_next, 1u);
                k = __shfl_sync(kFull, k, 0);
                if (k >= hi - lo) break;
                const uint32_t subj = hi - 1u - k;
                bool staged = staging && stage_issue(f, a, stage, 0, subj);
                if (staged && !stage_wait(f, a, 0)) {
                    // the copy never landed: read this and every later subject
                    // from global memory (the host reports the run as failed)
                    staging = false;
                    staged = false;
                }
                process_subject<QS, true>(f, a, c, q, subj, bq.index, staged ? stage : kNoStage, word_hits,
                                          residues);
            }
        }
        __syncthreads();
    }
    finish_counters(a, f, word_hits, residues);
}

}  // namespace

ScanLayout scan_layout(int32_t qlen, int32_t window, uint32_t stage_bytes, size_t smem_budget, int max_warps) {
    ScanLayout l{};
    l.diag_entries = static_cast<uint32_t>(qlen + window + 3) & ~3u;  // >= qlen + window
    l.diag_magic = static_cast<uint32_t>((1ull << 32) / l.diag_entries + 1);
    l.diag_bytes = l.diag_entries * 4u;
    l.stage_bytes = stage_bytes;
    l.query_smem_bytes = qlen <= kQuerySmemMax ? (static_cast<uint32_t>(qlen) + 15u) & ~15u : 0u;
    l.warp_smem_bytes = l.diag_bytes + 2 * kDeferCap * sizeof(uint2) + kSeedCap * sizeof(int4) + 16u +
                        ((stage_bytes + 32u + 15u) & ~15u);
    const size_t fixed = kScanMatBytes + kScanPresenceBytes + l.query_smem_bytes;
    int w = std::max(1, std::min(max_warps, kScanMaxWarpsPerBlock));
    while (w > 1 && fixed + static_cast<size_t>(w) * l.warp_smem_bytes > smem_budget) --w;
    l.warps_per_block = w;
    l.smem_bytes = fixed + static_cast<size_t>(w) * l.warp_smem_bytes;
    return l;
}

// Opts a scan kernel in to the device's full dynamic shared memory, once per
// (device, kernel). The attribute is process-wide: setting it per launch to
// that launch's size would let one host thread lower it between another
// thread's setting and launch, and that launch would then fail.
static cudaError_t allow_full_smem(const void *kernel) {
    static std::mutex mu;
    static std::set<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({dev, kernel})) return cudaSuccess;
    int optin = 0;
    cudaFuncAttributes fa{};
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // the dynamic allowance plus the kernel's static shared memory may not
    // exceed the opt-in limit
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - static_cast<int>(fa.sharedSizeBytes));
    if (e == cudaSuccess) done.insert({dev, kernel});
    return e;
}

cudaError_t launch_scan(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem_bytes, cudaStream_t st) {
    auto kernel = a.query_smem_bytes ? scan_kernel<true> : scan_kernel<false>;
    cudaError_t e = allow_full_smem(reinterpret_cast<const void *>(kernel));
    if (e != cudaSuccess) return e;
    kernel<<<n_blocks, warps_per_block * 32, smem_bytes, st>>>(a);
    return cudaGetLastError();
}

int scan_max_warps_by_registers(bool query_in_smem) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, query_in_smem ? scan_kernel<true> : scan_kernel<false>) != cudaSuccess)
        return kScanMaxWarpsPerBlock;
    int dev = 0, regs_per_block = 65536;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&regs_per_block, cudaDevAttrMaxRegistersPerBlock, dev);
    // registers are granted per warp in blocks of 256
    const int per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
    return per_warp > 0 ? std::max(1, std::min(kScanMaxWarpsPerBlock, std::min(fa.maxThreadsPerBlock / 32, regs_per_block / per_warp))) : kScanMaxWarpsPerBlock;
}

static void (*batch_kernel(bool query_in_smem))(ScanArgs) {
    return query_in_smem ? scan_batch_kernel<true> : scan_batch_kernel<false>;
}

cudaError_t launch_scan_batch(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem_bytes,
                              cudaStream_t st) {
    auto kernel = batch_kernel(a.query_smem_bytes != 0);
    cudaError_t e = allow_full_smem(reinterpret_cast<const void *>(kernel));
    if (e != cudaSuccess) return e;
    kernel<<<n_blocks, warps_per_block * 32, smem_bytes, st>>>(a);
    return cudaGetLastError();
}

cudaError_t scan_batch_occupancy(bool query_in_smem, int warps_per_block, size_t smem_bytes, int *blocks_per_sm) {
    auto kernel = batch_kernel(query_in_smem);
    cudaError_t e = allow_full_smem(reinterpret_cast<const void *>(kernel));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel, warps_per_block * 32, smem_bytes);
}

int scan_batch_max_warps_by_registers(bool query_in_smem) {
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, batch_kernel(query_in_smem)) != cudaSuccess) return kScanMaxWarpsPerBlock;
    int dev = 0, regs_per_block = 65536;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&regs_per_block, cudaDevAttrMaxRegistersPerBlock, dev);
    const int per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
    return per_warp > 0 ? std::max(1, std::min(kScanMaxWarpsPerBlock, std::min(fa.maxThreadsPerBlock / 32, regs_per_block / per_warp))) : kScanMaxWarpsPerBlock;
}

cudaError_t scan_occupancy(bool query_in_smem, int warps_per_block, size_t smem_bytes, int *blocks_per_sm) {
    auto kernel = query_in_smem ? scan_kernel<true> : scan_kernel<false>;
    cudaError_t e = allow_full_smem(reinterpret_cast<const void *>(kernel));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel, warps_per_block * 32,
                                                         smem_bytes);
}

}  // namespace blaze
