// kernels.cu -- the two device stages of the BLASTP preliminary search on
// GB300 (sm_103a). Integer work only: no tensor cores, no floating point.
//
//   scan_kernel    word lookup -> two-hit seeds (window 40) -> ungapped X-drop;
//                  one warp per subject, persistent warps pull subjects from a
//                  device cursor, longest first. Publishes the subject's
//                  ungapped HSPs (init hits) and a work item.
//   gapped_kernel  one warp per work item: orders the init hits, skips those
//                  contained in kept HSPs, runs the left and right score-only
//                  X-drop DP row-parallel across the warp, then purges common
//                  endpoints and sorts the subject's HSP list.
//
// Reference counterparts: gpuBLAZE_full (BLAZE_gpu/gpuBLAZE.cu:885-1252) and
// gpuBLAZE_everything (gpuBLAZE.cu:1254-1397); unlike those (a filter whose
// survivors the CPU re-searches) these produce the final HSPs.
#include <cstdint>

#include "common.cuh"

namespace blaze {

__device__ const int32_t g_blosum[kAlphabet * kAlphabet] = {
#include "blosum62.inc"
};

namespace {

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

__device__ __forceinline__ void load_matrix(int32_t *mat) {
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x) mat[i] = g_blosum[i];
}

// ------------------------------------------------------------------------
// Ungapped extension (scalar, one lane per seed). Same walks as the oracle:
// left from the end of the best word prefix, right only when the left walk
// reached the first hit (BLAZE_gpu/gpuBLAZE.cu:1096-1152 is the warp form).

__device__ int32_t extend_left(const uint8_t *__restrict__ q, const uint8_t *__restrict__ s,
                               int32_t q_off, int32_t s_off, int32_t xdrop, const int32_t *mat,
                               int32_t *length) {
    const int32_t n = min(s_off, q_off);
    int32_t best_i = n + 1, score = 0, maxscore = 0;
    const uint8_t *qq = q + q_off, *ss = s + s_off;
    for (int32_t k = 0; k <= n; ++k) {
        score += mat[qq[-k] * kAlphabet + ss[-k]];
        if (score > maxscore) {
            maxscore = score;
            best_i = n - k;
        }
        if (maxscore - score >= xdrop) break;
    }
    *length = n - best_i + 1;
    return maxscore;
}

__device__ int32_t extend_right(const uint8_t *__restrict__ q, int32_t qlen,
                                const uint8_t *__restrict__ s, int32_t slen, int32_t q_off,
                                int32_t s_off, int32_t xdrop, int32_t maxscore, const int32_t *mat,
                                int32_t *length, int32_t *s_last_off) {
    const int32_t n = min(slen - s_off, qlen - q_off);
    int32_t best_i = -1, score = maxscore, i;
    for (i = 0; i < n; ++i) {
        score += mat[q[q_off + i] * kAlphabet + s[s_off + i]];
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

__device__ int32_t extend_two_hit(const uint8_t *__restrict__ q, int32_t qlen,
                                  const uint8_t *__restrict__ s, int32_t slen, int32_t s_left_off,
                                  int32_t s_off, int32_t q_off, int32_t xdrop, const int32_t *mat,
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
// (s - q) mod table size, either the last recorded hit (biased by window and
// by a running base so the table never needs clearing between subjects),
// the same with kFlagBit after a right extension, or kPendBit | seed slot
// while that diagonal's extension is queued. A table of at least
// qlen + window entries cannot mix two diagonals that both matter.

struct WarpFinder {
    uint32_t *diag;
    uint2 *defer;     // two buffers of kDeferCap deferred hits {s, q}, arrival order
    int4 *seeds;      // {q, s, s_left_off, table index}
    int n_defer, n_seed, sel;
    uint32_t base;
    uint32_t n_init;
    const uint8_t *sub;
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
    const uint32_t d = static_cast<uint32_t>(s - q) & a.diag_mask;
    if (__ballot_sync(kFull, valid) == 0) return;
    const unsigned lt = lanemask_lt();
    const unsigned peers = __match_any_sync(kFull, valid ? d : 0xffffffffu);
    const unsigned rank = valid ? __popc(peers & lt) : 0u;
    const unsigned max_rank = __reduce_max_sync(kFull, rank);
    for (unsigned r = 0; r <= max_rank; ++r) {
        int act = kActNone;
        uint32_t newv = 0;
        int32_t s_left = 0;
        if (valid && rank == r) {
            const uint32_t e = wf.diag[d];
            if (e & kPendBit) {
                act = kActDefer;
            } else {
                const int32_t last = static_cast<int32_t>(e & kValMask) - a.window - static_cast<int32_t>(wf.base);
                if (e & kFlagBit) {
                    if (s >= last) {  // past the last extension: start over from this hit
                        act = kActSet;
                        newv = static_cast<uint32_t>(s + a.window) + wf.base;
                    }
                } else {
                    const int32_t diff = s - last;
                    if (diff >= a.window) {
                        act = kActSet;
                        newv = static_cast<uint32_t>(s + a.window) + wf.base;
                    } else if (diff >= kWordSize) {
                        act = kActSeed;
                        s_left = last + kWordSize;
                    }
                }
            }
        }
        const unsigned dm = __ballot_sync(kFull, act == kActDefer);
        if (act == kActDefer)
            wf.defer[wf.sel * kDeferCap + wf.n_defer + __popc(dm & lt)] = make_uint2(static_cast<uint32_t>(s), static_cast<uint32_t>(q));
        wf.n_defer += __popc(dm);
        const unsigned sm = __ballot_sync(kFull, act == kActSeed);
        if (act == kActSeed) {
            const int slot = wf.n_seed + __popc(sm & lt);
            wf.seeds[slot] = make_int4(q, s, s_left, static_cast<int32_t>(d));
            wf.diag[d] = kPendBit | static_cast<uint32_t>(slot);
        }
        wf.n_seed += __popc(sm);
        if (act == kActSet) wf.diag[d] = newv;
        __syncwarp();
    }
}

// Extends every queued seed (one lane each), settles their diagonals, keeps
// those reaching the ungapped cutoff, then replays the deferred hits; repeats
// until no seed and no deferred hit is left.
__device__ void flush(WarpFinder &wf, const ScanArgs &a, const int32_t *mat) {
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
                score = extend_two_hit(a.q, a.qlen, wf.sub, wf.slen, sd.z, sd.y, sd.x, a.xdrop, mat,
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
                    h.q_start = hq; h.s_start = hs; h.len = hl; h.score = score;
                    h.q_trig = sd.x; h.s_trig = sd.y;
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

__global__ void __launch_bounds__(kScanWarpsPerBlock * 32)
scan_kernel(const ScanArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    int32_t *mat = reinterpret_cast<int32_t *>(smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t entries = a.diag_mask + 1;
    const size_t per_warp = static_cast<size_t>(entries) * 4 + 2 * kDeferCap * sizeof(uint2) + kSeedCap * sizeof(int4);
    unsigned char *mine = smem + kAlphabet * kAlphabet * sizeof(int32_t) + warp * per_warp;
    load_matrix(mat);

    WarpFinder wf;
    wf.diag = reinterpret_cast<uint32_t *>(mine);
    wf.defer = reinterpret_cast<uint2 *>(mine + static_cast<size_t>(entries) * 4);
    wf.seeds = reinterpret_cast<int4 *>(wf.defer + 2 * kDeferCap);
    wf.n_defer = wf.n_seed = wf.sel = 0;
    wf.base = 0;
    wf.extensions = 0;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    wf.scratch = a.scratch + gwarp * a.scratch_cap;
    for (uint32_t i = lane; i < entries; i += 32) wf.diag[i] = 0;
    __syncthreads();

    unsigned long long word_hits = 0, residues = 0;
    const unsigned lt = lanemask_lt();
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_scan, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= a.n_subj) break;
        const uint32_t subj = a.n_subj - 1 - static_cast<uint32_t>(t);
        const uint64_t o0 = a.off[subj];
        wf.slen = static_cast<int32_t>(a.off[subj + 1] - o0);
        wf.sub = a.res + o0;
        wf.n_init = 0;
        residues += static_cast<unsigned long long>(wf.slen);
        const int32_t nwords = wf.slen - (kWordSize - 1);
        for (int32_t tb = 0; tb < nwords; tb += 32) {
            const int32_t p = tb + lane;
            uint32_t cs = 0, cnt = 0;
            if (p < nwords) {
                const int w = wf.sub[p] * 784 + wf.sub[p + 1] * 28 + wf.sub[p + 2];
                cs = __ldg(a.cell_start + w);
                cnt = __ldg(a.cell_start + w + 1) - cs;
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += x;
            }
            const uint32_t total = __shfl_sync(kFull, incl, 31);
            const uint32_t excl = incl - cnt;
            word_hits += total;
            for (uint32_t kb = 0; kb < total; kb += 32) {
                const uint32_t k = kb + lane;
                // owner = the last lane whose first hit index is <= k
                int lo = 0;
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const uint32_t ev = __shfl_sync(kFull, excl, lo + step);
                    if (ev <= k) lo += step;
                }
                const uint32_t hcs = __shfl_sync(kFull, cs, lo);
                const uint32_t hex = __shfl_sync(kFull, excl, lo);
                const bool hv = k < total;
                const int32_t qo = hv ? static_cast<int32_t>(__ldg(a.cell_off + hcs + (k - hex))) : 0;
                process_batch(wf, a, hv, tb + lo, qo);
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
        if (wf.base > kBaseReset) {
            __syncwarp();
            for (uint32_t i = lane; i < entries; i += 32) wf.diag[i] = 0;
            wf.base = 0;
        }
        __syncwarp();
    }
    (void)lt;
    if (lane == 0) {
        atomicAdd(&a.cnt->word_hits, word_hits);
        atomicAdd(&a.cnt->residues, residues);
        atomicAdd(&a.cnt->extensions, wf.extensions);
    }
}

// ------------------------------------------------------------------------
// Gapped stage.

__device__ __forceinline__ bool init_before(const InitHit &x, const InitHit &y) {
    if (x.score != y.score) return x.score > y.score;
    if (x.s_trig != y.s_trig) return x.s_trig < y.s_trig;
    return x.q_trig < y.q_trig;
}

__device__ int32_t gapped_start(const uint8_t *q, const uint8_t *s, int32_t q_start, int32_t s_start,
                                int32_t len, const int32_t *mat) {
    constexpr int32_t kWin = 11;  // gpuBLAZE.cu:1174-1208
    if (len <= kWin) return q_start + len / 2;
    int32_t score = 0;
    for (int32_t i = 0; i < kWin; ++i) score += mat[q[q_start + i] * kAlphabet + s[s_start + i]];
    int32_t max_score = score, max_offset = q_start + kWin - 1;
    const int32_t diag = s_start - q_start;
    for (int32_t i = q_start + kWin; i < q_start + len; ++i) {
        score -= mat[q[i - kWin] * kAlphabet + s[i - kWin + diag]];
        score += mat[q[i] * kAlphabet + s[i + diag]];
        if (score > max_score) {
            max_score = score;
            max_offset = i;
        }
    }
    return max_score > 0 ? max_offset - kWin / 2 : q_start;
}

// Score-only X-drop DP from the origin, computed one row at a time with the
// 32 lanes spread over the row's live columns. Row a, column b scores the
// a-th row letter against the b-th column letter (REV: both read backwards
// from the ends of A and B). Within a row the row-gap term and the running
// best are prefix maxima; a cell is live when it is within xdrop of the best
// seen so far in row-major order. Cells below that bound can never become
// live again, so computing the prefix maxima over every cell of the band
// (live or not) leaves all live values and the live set exactly those of the
// sequential band algorithm the oracle runs.
template <bool REV>
__device__ int32_t xdrop_dp(const uint8_t *__restrict__ A, const uint8_t *__restrict__ B, int32_t M,
                            int32_t N, int32_t gap_open, int32_t gap_extend, int32_t xdrop,
                            const int32_t *mat, int32_t *Hb, int32_t *Eb, int32_t *a_best,
                            int32_t *b_best, unsigned long long *cells) {
    const int lane = threadIdx.x & 31;
    const int32_t goe = gap_open + gap_extend, ge = gap_extend;
    if (xdrop < goe) xdrop = goe;
    *a_best = 0;
    *b_best = 0;
    if (M <= 0 || N <= 0) return 0;
    int32_t bsize = 1 + min(N, (xdrop - goe) / ge + 1);
    for (int32_t i = lane; i < bsize; i += 32) {
        const int32_t h = i == 0 ? 0 : -goe - (i - 1) * ge;
        Hb[i] = h;
        Eb[i] = h - goe;
    }
    __syncwarp();
    int32_t best = 0, first = 0, ab = 0, bb = 0;
    for (int32_t a = 1; a <= M; ++a) {
        const int32_t *row = mat + kAlphabet * (REV ? A[M - a] : A[a]);
        int32_t carry_p = kNeg, carry_best = best, carry_hold = kNeg;
        int32_t first_alive = -1, last_alive = -1, row_best = best, row_best_b = -1;
        *cells += static_cast<unsigned long long>(bsize - first);
        for (int32_t c0 = first; c0 < bsize; c0 += 32) {
            const int32_t b = c0 + lane;
            const bool act = b < bsize;
            const int32_t hold = act ? Hb[b] : kNeg;
            const int32_t ein = act ? Eb[b] : kNeg;
            int32_t hprev = __shfl_up_sync(kFull, hold, 1);
            if (lane == 0) hprev = carry_hold;
            int32_t D = ein;
            if (act && b > first) D = max(D, hprev + row[REV ? B[N - b] : B[b]]);
            const int32_t P = act ? max(D, kNeg) + ge * b : kNeg;
            int32_t incl = P;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t x = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl = max(incl, x);
            }
            int32_t excl = __shfl_up_sync(kFull, incl, 1);
            if (lane == 0) excl = kNeg;
            excl = max(excl, carry_p);
            const int32_t G = excl - goe + ge - ge * b;
            const int32_t H = max(D, G);
            int32_t inclh = act ? H : INT32_MIN;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t x = __shfl_up_sync(kFull, inclh, o);
                if (lane >= o) inclh = max(inclh, x);
            }
            int32_t exclh = __shfl_up_sync(kFull, inclh, 1);
            if (lane == 0) exclh = INT32_MIN;
            const int32_t cur_best = max(carry_best, exclh);
            const bool alive = act && (cur_best - H <= xdrop);
            const int32_t cm = __shfl_sync(kFull, inclh, 31);
            if (cm > carry_best) {
                const unsigned mm = __ballot_sync(kFull, act && H == cm);
                row_best = cm;
                row_best_b = c0 + __ffs(mm) - 1;
                carry_best = cm;
            }
            const unsigned am = __ballot_sync(kFull, alive);
            if (am) {
                if (first_alive < 0) first_alive = c0 + __ffs(am) - 1;
                last_alive = c0 + 31 - __clz(am);
            }
            carry_hold = __shfl_sync(kFull, hold, 31);
            carry_p = max(carry_p, __shfl_sync(kFull, incl, 31));
            __syncwarp();
            if (act) {
                if (alive) {
                    Eb[b] = max(H - goe, ein - ge);
                    Hb[b] = H;
                } else if (first_alive >= 0 && b > first_alive) {
                    Hb[b] = kNeg;
                }
            }
            __syncwarp();
        }
        if (first_alive < 0) break;
        if (row_best_b >= 0) {
            best = row_best;
            ab = a;
            bb = row_best_b;
        }
        first = first_alive;
        if (last_alive < bsize - 1) {
            bsize = last_alive + 1;
        } else {
            const int32_t F = carry_p - goe + ge - ge * bsize;
            const int32_t thr = best - xdrop;
            if (F >= thr && bsize <= N) {
                const int32_t n_ext = min(N - bsize + 1, (F - thr) / ge + 1);
                for (int32_t t = lane; t < n_ext; t += 32) {
                    Hb[bsize + t] = F - t * ge;
                    Eb[bsize + t] = F - t * ge - goe;
                }
                bsize += n_ext;
            }
        }
        if (bsize <= N) {
            if (lane == 0) {
                Hb[bsize] = kNeg;
                Eb[bsize] = kNeg;
            }
            ++bsize;
        }
        __syncwarp();
    }
    *a_best = ab;
    *b_best = bb;
    return best;
}

__device__ __forceinline__ int cmp_start(const DevHsp &a, const DevHsp &b) {
    if (a.q_start != b.q_start) return a.q_start < b.q_start ? -1 : 1;
    if (a.s_start != b.s_start) return a.s_start < b.s_start ? -1 : 1;
    if (a.score != b.score) return a.score > b.score ? -1 : 1;
    if (a.q_end != b.q_end) return a.q_end > b.q_end ? -1 : 1;
    if (a.s_end != b.s_end) return a.s_end > b.s_end ? -1 : 1;
    return 0;
}

__device__ __forceinline__ int cmp_end(const DevHsp &a, const DevHsp &b) {
    if (a.q_end != b.q_end) return a.q_end < b.q_end ? -1 : 1;
    if (a.s_end != b.s_end) return a.s_end < b.s_end ? -1 : 1;
    if (a.score != b.score) return a.score > b.score ? -1 : 1;
    if (a.q_start != b.q_start) return a.q_start < b.q_start ? -1 : 1;
    if (a.s_start != b.s_start) return a.s_start < b.s_start ? -1 : 1;
    return 0;
}

__device__ __forceinline__ int cmp_score(const DevHsp &a, const DevHsp &b) {
    if (a.score != b.score) return a.score > b.score ? -1 : 1;
    if (a.s_start != b.s_start) return a.s_start < b.s_start ? -1 : 1;
    if (a.s_end != b.s_end) return a.s_end > b.s_end ? -1 : 1;
    if (a.q_start != b.q_start) return a.q_start < b.q_start ? -1 : 1;
    if (a.q_end != b.q_end) return a.q_end > b.q_end ? -1 : 1;
    return 0;
}

template <int (*CMP)(const DevHsp &, const DevHsp &)>
__device__ void insertion_sort(DevHsp *h, int n) {
    for (int i = 1; i < n; ++i) {
        const DevHsp x = h[i];
        int j = i - 1;
        while (j >= 0 && CMP(x, h[j]) < 0) {
            h[j + 1] = h[j];
            --j;
        }
        h[j + 1] = x;
    }
}

// Drop HSPs sharing a start point, then an end point, with a better one;
// then order by score (one lane; lists are short).
__device__ int purge_and_sort(DevHsp *h, int n) {
    if (n <= 1) return n;
    insertion_sort<cmp_start>(h, n);
    int m = 0;
    for (int i = 0; i < n; ++i)
        if (m == 0 || h[i].q_start != h[m - 1].q_start || h[i].s_start != h[m - 1].s_start) h[m++] = h[i];
    n = m;
    insertion_sort<cmp_end>(h, n);
    m = 0;
    for (int i = 0; i < n; ++i)
        if (m == 0 || h[i].q_end != h[m - 1].q_end || h[i].s_end != h[m - 1].s_end) h[m++] = h[i];
    insertion_sort<cmp_score>(h, m);
    return m;
}

__global__ void __launch_bounds__(kGappedWarpsPerBlock * 32)
gapped_kernel(const GappedArgs a) {
    __shared__ int32_t mat[kAlphabet * kAlphabet];
    load_matrix(mat);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    InitHit *sorted = a.sorted + gwarp * a.cap;
    DevHsp *saved = a.saved + gwarp * a.cap;
    int32_t *Hb = a.dp + gwarp * 2ull * a.dp_stride;
    int32_t *Eb = Hb + a.dp_stride;
    unsigned long long n_work = *reinterpret_cast<volatile unsigned long long *>(&a.cnt->work_count);
    if (n_work > a.work_cap) n_work = a.work_cap;  // an overflowed run is repeated by the host
    unsigned long long cells = 0, n_ext = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_gapped, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= n_work) break;
        const WorkItem wi = a.work[t];
        const uint32_t n = wi.n_init;
        const InitHit *in = a.init_in + wi.first;
        const uint64_t o0 = a.off[wi.subject];
        const uint8_t *sub = a.res + o0;
        const int32_t slen = static_cast<int32_t>(a.off[wi.subject + 1] - o0);
        if (n > a.cap) {  // cannot happen: the scan kernel only publishes n <= its scratch cap
            if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadState);
            continue;
        }
        // order: score descending, ties in discovery order (rank sort)
        for (uint32_t i = lane; i < n; i += 32) {
            const InitHit hi = in[i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < n; ++j) rank += init_before(in[j], hi) ? 1u : 0u;
            sorted[rank] = hi;
        }
        __syncwarp();
        int nsaved = 0;
        for (uint32_t k = 0; k < n; ++k) {
            const InitHit u = sorted[k];
            bool inside = false;
            for (int j = lane; j < nsaved; j += 32) {
                const DevHsp g = saved[j];
                inside |= u.score <= g.score && g.q_start <= u.q_start && u.q_start + u.len <= g.q_end &&
                          g.s_start <= u.s_start && u.s_start + u.len <= g.s_end;
            }
            if (__any_sync(kFull, inside)) continue;
            int32_t q_off = 0;
            if (lane == 0) q_off = gapped_start(a.q, sub, u.q_start, u.s_start, u.len, mat);
            q_off = __shfl_sync(kFull, q_off, 0);
            const int32_t s_off = q_off + (u.s_start - u.q_start);
            int32_t al, bl, ar = 0, br = 0, right = 0;
            const int32_t left = xdrop_dp<true>(a.q, sub, q_off + 1, s_off + 1, a.gap_open, a.gap_extend,
                                                a.xdrop, mat, Hb, Eb, &al, &bl, &cells);
            if (q_off < a.qlen - 1 && s_off < slen - 1)
                right = xdrop_dp<false>(a.q + q_off, sub + s_off, a.qlen - q_off - 1, slen - s_off - 1,
                                        a.gap_open, a.gap_extend, a.xdrop, mat, Hb, Eb, &ar, &br, &cells);
            ++n_ext;
            const int32_t score = left + right;
            if (score >= a.cutoff) {
                if (lane == 0) {
                    DevHsp g;
                    g.subject = wi.subject;
                    g.score = score;
                    g.q_start = q_off + 1 - al;
                    g.q_end = q_off + ar + 1;
                    g.s_start = s_off + 1 - bl;
                    g.s_end = s_off + br + 1;
                    g.q_gs = q_off;
                    g.s_gs = s_off;
                    saved[nsaved] = g;
                }
                ++nsaved;
            }
            __syncwarp();
        }
        int m = 0;
        if (lane == 0) m = purge_and_sort(saved, nsaved);
        m = __shfl_sync(kFull, m, 0);
        __syncwarp();
        if (m > 0) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&a.cnt->out_count, static_cast<unsigned long long>(m));
            base = __shfl_sync(kFull, base, 0);
            if (base + m > a.out_cap) {
                if (lane == 0) atomicOr(&a.cnt->flags, kFlagOutArrayFull);
            } else {
                for (int i = lane; i < m; i += 32) a.out[base + i] = saved[i];
            }
        }
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->dp_cells, cells);
        atomicAdd(&a.cnt->gapped_ext, n_ext);
    }
}

}  // namespace

size_t scan_smem_bytes(uint32_t diag_entries, int warps_per_block) {
    const size_t per_warp = static_cast<size_t>(diag_entries) * 4 + 2 * kDeferCap * sizeof(uint2) + kSeedCap * sizeof(int4);
    return kAlphabet * kAlphabet * sizeof(int32_t) + per_warp * static_cast<size_t>(warps_per_block);
}

cudaError_t launch_scan(const ScanArgs &a, int n_blocks, int warps_per_block, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    scan_kernel<<<n_blocks, warps_per_block * 32, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gapped(const GappedArgs &a, int n_blocks, cudaStream_t st) {
    gapped_kernel<<<n_blocks, kGappedWarpsPerBlock * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t scan_occupancy(int warps_per_block, size_t smem, int *blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, scan_kernel,
                                                         warps_per_block * 32, smem);
}

cudaError_t gapped_occupancy(int *blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gapped_kernel,
                                                         kGappedWarpsPerBlock * 32, 0);
}

}  // namespace blaze
