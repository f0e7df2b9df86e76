// kernels.cu -- the gapped stage of the BLASTP preliminary search on GB300
// (sm_103a). Integer work only: no tensor cores, no floating point. (The
// word finder, two-hit and ungapped stage is scan.cu.)
//
//   gapped_kernel  one warp per work item: orders the init hits, skips those
//                  contained in kept HSPs, runs the left and right score-only
//                  X-drop DP row-parallel across the warp, then purges common
//                  endpoints, sorts the subject's HSP list and keeps what the
//                  preliminary reap and max_hsps keep.
//   hitlist_*      per query, the hitlist_size best subject lists (radix
//                  select on the device).
//
// Reference counterpart: gpuBLAZE_everything (BLAZE_gpu/gpuBLAZE.cu:1254-1397);
// unlike that filter (whose survivors the CPU re-searches) this kernel
// produces the final HSPs.
#include <algorithm>
#include <mutex>
#include <cstdint>

#include "common.cuh"

namespace blaze {

__device__ const int32_t g_blosum[kAlphabet * kAlphabet] = {
#include "blosum62.inc"
};

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void load_matrix(int32_t *mat) {
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x) mat[i] = g_blosum[i];
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
// warp spread over the row's live columns, two adjacent columns per lane (64
// per step: most rows of a band are 33 to 64 wide, so a row is one step).
// Row a, column b scores the a-th row letter against the b-th column letter
// (REV: both read backwards from the ends of A and B). Within a row the
// row-gap term and the running best are prefix maxima (within the lane's
// pair, then across lanes); a cell is live when it is within xdrop of the
// best seen so far in row-major order. Cells below that bound can never
// become live again, so computing the prefix maxima over every cell of the
// band (live or not) leaves all live values and the live set exactly those
// of the sequential band algorithm the oracle runs. The running best's prefix
// maximum is taken only in a step whose largest value beats the best carried
// into it (a warp max-reduce decides); in every other step the carried best
// is each cell's best so far. Hb and Eb are 8-byte aligned and hold at least
// N + 2 entries, so the pair loads and stores of a live column stay inside.
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
        for (int32_t c0 = first & ~1; c0 < bsize; c0 += 64) {
            const int32_t b0 = c0 + 2 * lane, b1 = b0 + 1;
            const bool act0 = b0 >= first && b0 < bsize, act1 = b1 >= first && b1 < bsize;
            int2 hold = make_int2(kNeg, kNeg), ein = make_int2(kNeg, kNeg);
            if (b0 < bsize) {  // b1 <= bsize <= N + 1: inside the rows
                hold = *reinterpret_cast<const int2 *>(Hb + b0);
                ein = *reinterpret_cast<const int2 *>(Eb + b0);
            }
            if (!act0) hold.x = ein.x = kNeg;
            if (!act1) hold.y = ein.y = kNeg;
            int32_t hprev = __shfl_up_sync(kFull, hold.y, 1);
            if (lane == 0) hprev = carry_hold;
            int32_t D0 = ein.x, D1 = ein.y;
            if (act0 && b0 > first) D0 = __viaddmax_s32(hprev, row[REV ? B[N - b0] : B[b0]], D0);
            if (act1 && b1 > first) D1 = __viaddmax_s32(hold.x, row[REV ? B[N - b1] : B[b1]], D1);
            const int32_t P0 = act0 ? max(D0, kNeg) + ge * b0 : kNeg;
            const int32_t P1 = act1 ? max(D1, kNeg) + ge * b1 : kNeg;
            // row gap: prefix maximum of P over the columns before each cell
            int32_t incl = max(P0, P1);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) incl = max(incl, __shfl_up_sync(kFull, incl, o));  // lanes < o get their own
            int32_t excl = __shfl_up_sync(kFull, incl, 1);
            if (lane == 0) excl = kNeg;
            excl = max(excl, carry_p);
            const int32_t G0 = excl - goe + ge - ge * b0;
            const int32_t G1 = max(excl, P0) - goe + ge - ge * b1;
            const int32_t H0 = max(D0, G0), H1 = max(D1, G1);
            // the best so far in row-major order: only a step whose largest
            // H beats the carried best needs the prefix maximum
            const int32_t hv0 = act0 ? H0 : INT32_MIN, hv1 = act1 ? H1 : INT32_MIN;
            const int32_t cm = __reduce_max_sync(kFull, max(hv0, hv1));
            int32_t best0 = carry_best, best1 = carry_best;
            if (cm > carry_best) {
                int32_t inclh = max(hv0, hv1);
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) inclh = max(inclh, __shfl_up_sync(kFull, inclh, o));
                int32_t exclh = __shfl_up_sync(kFull, inclh, 1);
                if (lane == 0) exclh = INT32_MIN;
                best0 = max(carry_best, exclh);
                best1 = max(best0, hv0);
                const unsigned m0 = __ballot_sync(kFull, act0 && H0 == cm);
                const unsigned m1 = __ballot_sync(kFull, act1 && H1 == cm);
                const int f0 = m0 ? 2 * (__ffs(m0) - 1) : 64, f1 = m1 ? 2 * (__ffs(m1) - 1) + 1 : 64;
                row_best = cm;
                row_best_b = c0 + min(f0, f1);
                carry_best = cm;
            }
            const bool alive0 = act0 && (best0 - H0 <= xdrop);
            const bool alive1 = act1 && (best1 - H1 <= xdrop);
            const unsigned a0 = __ballot_sync(kFull, alive0), a1 = __ballot_sync(kFull, alive1);
            if (a0 | a1) {
                const int f0 = a0 ? 2 * (__ffs(a0) - 1) : 64, f1 = a1 ? 2 * (__ffs(a1) - 1) + 1 : 64;
                const int l0 = a0 ? 2 * (31 - __clz(a0)) : -1, l1 = a1 ? 2 * (31 - __clz(a1)) + 1 : -1;
                if (first_alive < 0) first_alive = c0 + min(f0, f1);
                last_alive = c0 + max(l0, l1);
            }
            carry_hold = __shfl_sync(kFull, hold.y, 31);
            carry_p = max(carry_p, __shfl_sync(kFull, incl, 31));
            __syncwarp();
            if (act0) {
                if (alive0) {
                    Eb[b0] = __viaddmax_s32(H0, -goe, ein.x - ge);
                    Hb[b0] = H0;
                } else if (first_alive >= 0 && b0 > first_alive) {
                    Hb[b0] = kNeg;
                }
            }
            if (act1) {
                if (alive1) {
                    Eb[b1] = __viaddmax_s32(H1, -goe, ein.y - ge);
                    Hb[b1] = H1;
                } else if (first_alive >= 0 && b1 > first_alive) {
                    Hb[b1] = kNeg;
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

// One work item of the gapped stage, read and checked.
struct Item {
    WorkItem wi;
    uint32_t qi;
    const uint8_t *qres, *sub;
    int32_t qlen, slen, cutoff, smin, max_hsps;
    uint32_t n;
    const InitHit *in;
};

// Reads work item t; false when it must be skipped (a flag is then set).
__device__ __forceinline__ bool read_item(const GappedArgs &a, unsigned long long t, Item &it, int lane) {
    it.wi = a.work[t];
    it.qi = a.work_query ? a.work_query[t] : 0u;
    const WorkItem &wi = it.wi;
    if (wi.subject >= a.n_subj || it.qi >= a.n_queries || wi.first > a.init_cap ||
        wi.n_init > a.init_cap - wi.first) {  // cannot happen: every counted item is written
        if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadState);
        return false;
    }
    it.qres = a.work_query ? a.batch_q[it.qi] : a.q;
    it.qlen = a.work_query ? a.batch_qlen[it.qi] : a.qlen;
    it.cutoff = a.work_query ? a.batch_cutoff[it.qi] : a.cutoff;
    it.smin = a.work_query ? a.batch_smin[it.qi] : a.smin;
    it.max_hsps = a.work_query ? a.batch_max_hsps[it.qi] : a.max_hsps;
    it.n = wi.n_init;
    it.in = a.init_in + wi.first;
    const uint64_t o0 = a.off[wi.subject];
    const uint64_t o1 = a.off[wi.subject + 1];
    it.sub = a.res + o0;
    if (it.n > a.cap) {  // cannot happen: the scan kernel only publishes n <= its scratch cap
        if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadState);
        return false;
    }
    // The DP rows hold dp_stride ints: a subject too long for them (only
    // possible where the caller sized the rows, as the allocation-free
    // entry point does) is skipped and reported.
    if (o1 < o0 || o1 - o0 + 2u > a.dp_stride) {
        if (lane == 0) atomicOr(&a.cnt->flags, kFlagSubjectTooLong);
        return false;
    }
    it.slen = static_cast<int32_t>(o1 - o0);
    return true;
}

// Orders the item's init hits into dst: score descending, ties in discovery
// order (rank sort; equal records, which only a caller can pass, keep their
// input order, so every slot is written).
__device__ __forceinline__ void order_init_hits(const Item &it, InitHit *dst, int lane) {
    const uint32_t n = it.n;
    for (uint32_t i = lane; i < n; i += 32) {
        const InitHit hi = it.in[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) {
            const InitHit hj = it.in[j];
            rank += (init_before(hj, hi) || (j < i && !init_before(hi, hj))) ? 1u : 0u;
        }
        dst[rank] = hi;
    }
    __syncwarp();
}

// An init hit must lie inside the query and the subject (the scan kernel's
// always do; a caller's may not).
__device__ __forceinline__ bool init_hit_inside(const InitHit &u, const Item &it) {
    return !(u.len < 1 || u.q_start < 0 || u.s_start < 0 || u.len > it.qlen - u.q_start ||
             u.len > it.slen - u.s_start);
}

// Whether init hit u lies inside a kept HSP scoring at least as much.
__device__ __forceinline__ bool contained(const InitHit &u, const DevHsp *saved, int nsaved, int lane) {
    bool inside = false;
    for (int j = lane; j < nsaved; j += 32) {
        const DevHsp g = saved[j];
        inside |= u.score <= g.score && g.q_start <= u.q_start && u.q_start + u.len <= g.q_end &&
                  g.s_start <= u.s_start && u.s_start + u.len <= g.s_end;
    }
    return __any_sync(kFull, inside);
}

__device__ __forceinline__ DevHsp make_hsp(uint32_t subject, int32_t score, int32_t q_off, int32_t s_off,
                                           int32_t al, int32_t bl, int32_t ar, int32_t br) {
    DevHsp g;
    g.subject = subject;
    g.score = score;
    g.q_start = q_off + 1 - al;
    g.q_end = q_off + ar + 1;
    g.s_start = s_off + 1 - bl;
    g.s_end = s_off + br + 1;
    g.q_gs = q_off;
    g.s_gs = s_off;
    return g;
}

// Purges and orders the item's kept HSPs, applies the preliminary E-value
// reap (E-values fall with the score, so it keeps the leading HSPs scoring
// at least smin) and max_hsps, and publishes the list.
__device__ __forceinline__ void publish(const GappedArgs &a, const Item &it, DevHsp *saved, int nsaved, int lane) {
    int m = 0;
    if (lane == 0) {
        const int all = purge_and_sort(saved, nsaved);
        while (m < all && saved[m].score >= it.smin) ++m;
        if (it.max_hsps > 0 && m > it.max_hsps) m = it.max_hsps;
    }
    m = __shfl_sync(kFull, m, 0);
    __syncwarp();
    if (m == 0) return;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&a.cnt->out_count, static_cast<unsigned long long>(m));
    base = __shfl_sync(kFull, base, 0);
    if (base + m > a.out_cap) {
        if (lane == 0) atomicOr(&a.cnt->flags, kFlagOutArrayFull);
        return;
    }
    for (int i = lane; i < m; i += 32) a.out[base + i] = saved[i];
    if (lane == 0 && a.groups) {
        // every published list holds at least one of the out_cap HSPs, so
        // the descriptor index stays below out_cap
        const unsigned long long gi = atomicAdd(&a.cnt->group_count, 1ull);
        GroupDesc g;
        g.first = base;
        g.query = it.qi;
        g.subject = it.wi.subject;
        g.oid = a.oid[it.wi.subject];
        g.n = static_cast<uint32_t>(m);
        g.best = saved[0].score;
        g.pad = 0;
        a.groups[gi] = g;
        if (a.qkept) atomicAdd(&a.qkept[it.qi], 1u);
    }
}

// Number of work items this pass may take: none when the scan overflowed
// its init-hit or work array (the host repeats that pass with larger
// arrays, and an unwritten slot holds no valid item).
__device__ __forceinline__ unsigned long long work_items(const GappedArgs &a) {
    unsigned long long n_work = *reinterpret_cast<volatile unsigned long long *>(&a.cnt->work_count);
    if (n_work > a.work_cap) n_work = a.work_cap;
    const unsigned scan_flags = *reinterpret_cast<volatile unsigned *>(&a.cnt->flags);
    if (scan_flags & (kFlagInitArrayFull | kFlagWorkArrayFull | kFlagBadState)) n_work = 0;
    return n_work;
}

// The whole gapped stage in one kernel, one warp per work item (single
// queries, small batches and the allocation-free entry point).
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
    if (n_work > a.work_cap) n_work = a.work_cap;
    // A scan that overflowed its init-hit or work array counted items it
    // could not write; the host repeats that pass with larger arrays, so this
    // one takes no work at all (an unwritten slot holds no valid item).
    const unsigned scan_flags = *reinterpret_cast<volatile unsigned *>(&a.cnt->flags);
    if (scan_flags & (kFlagInitArrayFull | kFlagWorkArrayFull | kFlagBadState)) n_work = 0;
    unsigned long long cells = 0, n_ext = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_gapped, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= n_work) break;
        const WorkItem wi = a.work[t];
        const uint32_t qi = a.work_query ? a.work_query[t] : 0u;
        if (wi.subject >= a.n_subj || qi >= a.n_queries || wi.first > a.init_cap ||
            wi.n_init > a.init_cap - wi.first) {  // cannot happen: every counted item is written
            if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadState);
            continue;
        }
        const uint8_t *qres = a.work_query ? a.batch_q[qi] : a.q;
        const int32_t qlen = a.work_query ? a.batch_qlen[qi] : a.qlen;
        const int32_t cutoff = a.work_query ? a.batch_cutoff[qi] : a.cutoff;
        const int32_t smin = a.work_query ? a.batch_smin[qi] : a.smin;
        const int32_t max_hsps = a.work_query ? a.batch_max_hsps[qi] : a.max_hsps;
        const uint32_t n = wi.n_init;
        const InitHit *in = a.init_in + wi.first;
        const uint64_t o0 = a.off[wi.subject];
        const uint8_t *sub = a.res + o0;
        const uint64_t o1 = a.off[wi.subject + 1];
        if (n > a.cap) {  // cannot happen: the scan kernel only publishes n <= its scratch cap
            if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadState);
            continue;
        }
        // The DP rows hold dp_stride ints: a subject too long for them (only
        // possible where the caller sized the rows, as the allocation-free
        // entry point does) is skipped and reported.
        if (o1 < o0 || o1 - o0 + 2u > a.dp_stride) {
            if (lane == 0) atomicOr(&a.cnt->flags, kFlagSubjectTooLong);
            continue;
        }
        const int32_t slen = static_cast<int32_t>(o1 - o0);
        // order: score descending, ties in discovery order (rank sort; equal
        // records, which only a caller can pass, keep their input order, so
        // every slot is written)
        for (uint32_t i = lane; i < n; i += 32) {
            const InitHit hi = in[i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < n; ++j) {
                const InitHit hj = in[j];
                rank += (init_before(hj, hi) || (j < i && !init_before(hi, hj))) ? 1u : 0u;
            }
            sorted[rank] = hi;
        }
        __syncwarp();
        int nsaved = 0;
        for (uint32_t k = 0; k < n; ++k) {
            const InitHit u = sorted[k];
            // an init hit must lie inside the query and the subject (the scan
            // kernel's always do; a caller's may not): others are skipped
            if (u.len < 1 || u.q_start < 0 || u.s_start < 0 || u.len > qlen - u.q_start ||
                u.len > slen - u.s_start) {
                if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadInitHit);
                continue;
            }
            bool inside = false;
            for (int j = lane; j < nsaved; j += 32) {
                const DevHsp g = saved[j];
                inside |= u.score <= g.score && g.q_start <= u.q_start && u.q_start + u.len <= g.q_end &&
                          g.s_start <= u.s_start && u.s_start + u.len <= g.s_end;
            }
            if (__any_sync(kFull, inside)) continue;
            int32_t q_off = 0;
            if (lane == 0) q_off = gapped_start(qres, sub, u.q_start, u.s_start, u.len, mat);
            q_off = __shfl_sync(kFull, q_off, 0);
            const int32_t s_off = q_off + (u.s_start - u.q_start);
            int32_t al, bl, ar = 0, br = 0, right = 0;
            const int32_t left = xdrop_dp<true>(qres, sub, q_off + 1, s_off + 1, a.gap_open, a.gap_extend,
                                                a.xdrop, mat, Hb, Eb, &al, &bl, &cells);
            if (q_off < qlen - 1 && s_off < slen - 1)
                right = xdrop_dp<false>(qres + q_off, sub + s_off, qlen - q_off - 1, slen - s_off - 1,
                                        a.gap_open, a.gap_extend, a.xdrop, mat, Hb, Eb, &ar, &br, &cells);
            ++n_ext;
            const int32_t score = left + right;
            if (score >= cutoff) {
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
        // purge and order; then the preliminary E-value reap (E-values fall
        // with the score, so it keeps the leading HSPs scoring at least smin)
        // and at most max_hsps of them
        int m = 0;
        if (lane == 0) {
            const int all = purge_and_sort(saved, nsaved);
            while (m < all && saved[m].score >= smin) ++m;
            if (max_hsps > 0 && m > max_hsps) m = max_hsps;
        }
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
                if (lane == 0 && a.groups) {
                    // every published list holds at least one of the out_cap
                    // HSPs, so the descriptor index stays below out_cap
                    const unsigned long long gi = atomicAdd(&a.cnt->group_count, 1ull);
                    GroupDesc g;
                    g.first = base;
                    g.query = qi;
                    g.subject = wi.subject;
                    g.oid = a.oid[wi.subject];
                    g.n = static_cast<uint32_t>(m);
                    g.best = saved[0].score;
                    g.pad = 0;
                    a.groups[gi] = g;
                    if (a.qkept) atomicAdd(&a.qkept[qi], 1u);
                }
            }
        }
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->dp_cells, cells);
        atomicAdd(&a.cnt->gapped_ext, n_ext);
    }
}

// ------------------------------------------------------------------------
// The gapped stage in three kernels, for batched passes of many queries:
//
//   gapped_prep_kernel    one warp per work item: orders its init hits into
//                         the pass-wide init_sorted array (same slots as the
//                         scan wrote them) and writes one DP task per init
//                         hit (its gapped start point);
//   gapped_dp_kernel      one LANE per X-drop DP (the left and the right one
//                         of every init hit): each lane runs the sequential
//                         banded X-drop of the oracle on its own task, rows of
//                         the warp's 32 tasks in step, its DP row in a
//                         shared-memory ring of kDpRing columns; a task whose
//                         band gets wider than the ring is left to the
//                         finishing kernel;
//   gapped_finish_kernel  one warp per work item: walks the ordered init
//                         hits, skips those inside kept HSPs (so the DPs of
//                         skipped init hits, computed ahead, go unused),
//                         takes the DP results (running the warp-parallel DP
//                         for a task the lane kernel left), and publishes.
//
// Every DP is independent of the others (containment only decides which
// results are used), so the results are exactly those of gapped_kernel.

__global__ void __launch_bounds__(kGappedWarpsPerBlock * 32)
gapped_prep_kernel(const GappedArgs a) {
    __shared__ int32_t mat[kAlphabet * kAlphabet];
    load_matrix(mat);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned long long n_work = work_items(a);
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_prep, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= n_work) break;
        Item it;
        const bool ok = read_item(a, t, it, lane);
        const WorkItem wi = a.work[t];
        if (!ok) {
            // its tasks stay empty (the checks bounded n_init by init_cap)
            if (wi.first <= a.init_cap && wi.n_init <= a.init_cap - wi.first)
                for (uint32_t k = lane; k < wi.n_init; k += 32) a.dtask[wi.first + k].valid = 0;
            continue;
        }
        InitHit *dst = a.init_sorted + wi.first;
        order_init_hits(it, dst, lane);
        for (uint32_t k = lane; k < it.n; k += 32) {
            const InitHit u = dst[k];
            DpTask d;
            d.s_base = a.off[wi.subject];
            d.slen = it.slen;
            d.query = it.qi;
            d.q_off = 0;
            d.s_off = 0;
            d.valid = init_hit_inside(u, it) ? 1 : 0;
            d.pad = 0;
            if (d.valid) {
                d.q_off = gapped_start(it.qres, it.sub, u.q_start, u.s_start, u.len, mat);
                d.s_off = d.q_off + (u.s_start - u.q_start);
            }
            a.dtask[wi.first + k] = d;
        }
    }
}

// Packed DP cell of the lane kernel's ring: H (21 bits, signed; |H| stays
// below 2^20, tasks that could score more go to the warp-parallel DP), a
// dead flag (H is -inf), d = H - gap_extend - E (5 bits: for a cell written
// live, H - gap_open - gap_extend <= E <= H - gap_extend) and the letter of
// the NEXT column (5 bits), which the diagonal move into it scores.
constexpr int kDpRing = 64;            // ring columns per lane (a power of 2)
constexpr int kDpWarpsPerBlock = 4;
constexpr int32_t kDpHMax = (1 << 20) - 64;
constexpr uint32_t kDpDead = 1u << 10;

__device__ __forceinline__ uint32_t dp_pack(int32_t h, int32_t e, int32_t ge, uint32_t letter) {
    return (static_cast<uint32_t>(h) << 11) | (static_cast<uint32_t>(h - ge - e) << 5) | letter;
}
// H = -inf and E = -inf: the H field holds -2^20 and d = 31, so E decodes
// below every score a band can reach
__device__ __forceinline__ uint32_t dp_pack_inf(uint32_t letter) {
    return (static_cast<uint32_t>(-(1 << 20)) << 11) | kDpDead | (31u << 5) | letter;
}

struct DpConsts {
    int32_t ge, goe, xdrop, bsize0;
};

// One lane's task: rows are query letters, columns subject letters, read
// forwards (right extension) or backwards (left extension) from the start.
struct DpLane {
    bool has;
    unsigned long long t;
    const uint8_t *S, *Q;  // letter k of the row / column sequence is at [dir * k]
    int32_t dir, M, N;
    int32_t row, first, bsize, best, ab, bb, cells, thr, rowoff;
};

__device__ __forceinline__ void dp_lane_start(DpLane &L, unsigned long long t, const GappedArgs &a,
                                              const DpConsts &c, uint32_t *R) {
#define RS(x) R[((x) & (kDpRing - 1)) * 32]
    L.t = t;
    L.has = false;
    const DpTask k = a.dtask[t >> 1];
    const bool left = (t & 1ull) == 0;
    const uint8_t *q = a.work_query ? a.batch_q[k.query] : a.q;
    const int32_t qlen = a.work_query ? a.batch_qlen[k.query] : a.qlen;
    const uint64_t total = a.off[a.n_subj];
    // a record is checked before use (every slot is written by the prep
    // kernel; a stale one from another pass must not send reads astray)
    if (!k.valid || k.query >= a.n_queries || k.s_base > total || static_cast<uint64_t>(k.slen) > total - k.s_base ||
        k.q_off < 0 || k.q_off >= qlen || k.s_off < 0 || k.s_off >= k.slen) {
        if (k.valid) atomicOr(&a.cnt->flags, kFlagBadState);
        a.dres[t] = make_int4(0, 0, 0, 0);
        return;
    }
    const uint8_t *sb = a.res + k.s_base;
    int32_t M, N;
    if (left) {
        L.dir = -1; L.S = sb + k.s_off + 1; L.Q = q + k.q_off + 1; M = k.q_off + 1; N = k.s_off + 1;
    } else {
        L.dir = 1; L.S = sb + k.s_off; L.Q = q + k.q_off; M = qlen - k.q_off - 1; N = k.slen - k.s_off - 1;
    }
    L.M = M;
    L.N = N;
    if (M <= 0 || N <= 0) {
        a.dres[t] = make_int4(0, 0, 0, 0);
        return;
    }
    const int32_t bs = N + 1 < c.bsize0 ? N + 1 : c.bsize0;
    // the packed cell holds H within +-2^20 (BLOSUM62 scores at most 11 per
    // cell, live cells stay above -xdrop) and d <= 31 (gap_open <= 31)
    if (bs > kDpRing || 11ll * (M < N ? M : N) >= kDpHMax || c.xdrop >= kDpHMax || c.goe - c.ge > 31) {
        a.dres[t] = make_int4(0, 0, 0, -1);
        return;
    }
    for (int32_t j = 0; j < bs; ++j) {
        const int32_t hv = j == 0 ? 0 : -c.goe - (j - 1) * c.ge;
        const uint32_t letter = j + 1 <= N ? L.S[L.dir * (j + 1)] : 0u;
        RS(j) = dp_pack(hv, hv - c.goe, c.ge, letter);
    }
    L.bsize = bs;
    L.first = 0;
    L.row = 1;
    L.best = L.ab = L.bb = 0;
    L.cells = bs;
    L.thr = -c.xdrop;
    L.rowoff = kAlphabet * static_cast<int32_t>(L.Q[L.dir]);
    L.has = true;
}

// The lane's current row: its cells in a tight loop (the sequential band
// algorithm of the oracle, cell by cell), then the row's end.
__device__ __forceinline__ void dp_lane_row(DpLane &L, const GappedArgs &a, const DpConsts &c, const int32_t *mat,
                                            uint32_t *R) {
    int32_t b = L.first, first = L.first, last = L.first;
    const int32_t bsize = L.bsize, N = L.N, row = L.row, rowoff = L.rowoff;
    int32_t h = kNeg, f = kNeg, best = L.best, thr = L.thr, ab = L.ab, bb = L.bb;
    uint32_t p = RS(b);
    for (; b < bsize; ++b) {
        const uint32_t p_n = RS(b + 1);
        const uint32_t lt = p & 31u;
        const int32_t hl = static_cast<int32_t>(p) >> 11;
        const int32_t e = hl - c.ge - static_cast<int32_t>((p >> 5) & 31u);
        const int32_t hb = (p & kDpDead) ? kNeg : hl;
        const int32_t sc = mat[rowoff + static_cast<int32_t>(lt)];
        const int32_t hh = max(max(h, e), f);
        const bool alive = hh >= thr;
        const bool up = hh > best;
        best = up ? hh : best;
        ab = up ? row : ab;
        bb = up ? b : bb;
        thr = up ? hh - c.xdrop : thr;
        const int32_t eo = hh - c.goe;
        const int32_t en = max(eo, e - c.ge);
        f = alive ? max(eo, f - c.ge) : f;
        last = alive ? b : last;
        const bool lead = !alive && b == first;
        first += lead ? 1 : 0;
        if (!lead) RS(b) = alive ? dp_pack(hh, en, c.ge, lt) : (p | kDpDead);
        h = b + 1 <= N ? hb + sc : kNeg;
        p = p_n;
    }
    L.best = best;
    L.thr = thr;
    L.ab = ab;
    L.bb = bb;
    L.first = first;
    if (first == bsize) {  // no live cell in the row
        a.dres[L.t] = make_int4(best, ab, bb, L.cells);
        L.has = false;
        return;
    }
    int32_t bs = bsize;
    if (last < bs - 1) {
        // the band ends after its last live cell; that next column's H is
        // already -inf (a dead cell of this row): make its E -inf too
        bs = last + 1;
        if (bs <= N) {
            RS(bs) = dp_pack_inf(RS(bs) & 31u);
            bs++;
        }
    } else {
        bool ovf = false;
        while (f >= thr && bs <= N) {  // the row ended live: extend along its row gap
            if (bs + 1 - first > kDpRing) { ovf = true; break; }
            const uint32_t letter = bs + 1 <= N ? L.S[L.dir * (bs + 1)] : 0u;
            RS(bs) = dp_pack(f, f - c.goe, c.ge, letter);
            f -= c.ge;
            bs++;
        }
        if (!ovf && bs <= N) {
            if (bs + 1 - first > kDpRing) {
                ovf = true;
            } else {
                const uint32_t letter = bs + 1 <= N ? L.S[L.dir * (bs + 1)] : 0u;
                RS(bs) = dp_pack_inf(letter);
                bs++;
            }
        }
        if (ovf) {  // the band outgrew the ring: the finishing kernel reruns this DP
            a.dres[L.t] = make_int4(0, 0, 0, -1);
            L.has = false;
            return;
        }
    }
    L.bsize = bs;
    L.row = row + 1;
    if (L.row > L.M) {
        a.dres[L.t] = make_int4(best, ab, bb, L.cells);
        L.has = false;
        return;
    }
    L.rowoff = kAlphabet * static_cast<int32_t>(L.Q[L.dir * L.row]);
    L.cells += bs - first;
#undef RS
}

// Tasks reach a warp in chunks of 32 from a pass-wide cursor (lane 0 takes
// the next chunk's index ahead); the lanes that need a task take the next
// ones of the chunk.
__global__ void __launch_bounds__(kDpWarpsPerBlock * 32)
gapped_dp_kernel(const GappedArgs a) {
    __shared__ int32_t mat[kAlphabet * kAlphabet];
    extern __shared__ __align__(16) uint32_t dp_smem[];
    load_matrix(mat);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t *R = dp_smem + wib * (kDpRing * 32) + lane;
    DpConsts c;
    c.ge = a.gap_extend;
    c.goe = a.gap_open + a.gap_extend;
    c.xdrop = a.xdrop < c.goe ? c.goe : a.xdrop;
    c.bsize0 = 1 + (c.xdrop - c.goe) / c.ge + 1;
    unsigned long long n_init = 0;
    {
        n_init = *reinterpret_cast<volatile unsigned long long *>(&a.cnt->init_count);
        if (n_init > a.init_cap) n_init = a.init_cap;
        if (work_items(a) == 0) n_init = 0;
    }
    const unsigned long long n = 2ull * n_init;
    unsigned long long next = 0, cur;
    if (lane == 0) next = atomicAdd(&a.cnt->next_dp, 32ull);
    cur = __shfl_sync(kFull, next, 0);
    int32_t cnt = cur < n ? static_cast<int32_t>(n - cur < 32ull ? n - cur : 32ull) : 0, qpos = 0;
    if (lane == 0) next = atomicAdd(&a.cnt->next_dp, 32ull);
    DpLane L;
    L.has = false;
    for (;;) {
        unsigned need = __ballot_sync(kFull, !L.has);
        while (need) {
            if (qpos >= cnt) {  // the next chunk
                cur = __shfl_sync(kFull, next, 0);
                cnt = cur < n ? static_cast<int32_t>(n - cur < 32ull ? n - cur : 32ull) : 0;
                qpos = 0;
                if (lane == 0 && cur < n) next = atomicAdd(&a.cnt->next_dp, 32ull);
            }
            const int32_t idx = qpos + __popc(need & lanemask_lt());
            qpos += __popc(need);
            if (!L.has && idx < cnt) dp_lane_start(L, cur + idx, a, c, R);
            if (cnt == 0) break;  // no task left for anyone
            need = __ballot_sync(kFull, !L.has);
        }
        if (__ballot_sync(kFull, L.has) == 0) break;
        if (L.has) dp_lane_row(L, a, c, mat, R);
    }
}

__global__ void __launch_bounds__(kGappedWarpsPerBlock * 32)
gapped_finish_kernel(const GappedArgs a) {
    __shared__ int32_t mat[kAlphabet * kAlphabet];
    load_matrix(mat);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    DevHsp *saved = a.saved + gwarp * a.cap;
    int32_t *Hb = a.dp + gwarp * 2ull * a.dp_stride;
    int32_t *Eb = Hb + a.dp_stride;
    const unsigned long long n_work = work_items(a);
    unsigned long long cells = 0, n_ext = 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&a.cnt->next_gapped, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= n_work) break;
        Item it;
        if (!read_item(a, t, it, lane)) continue;  // flagged by the prep kernel already
        const InitHit *sorted = a.init_sorted + it.wi.first;
        const DpTask *tasks = a.dtask + it.wi.first;
        const int4 *res = a.dres + 2ull * it.wi.first;
        int nsaved = 0;
        for (uint32_t k = 0; k < it.n; ++k) {
            const InitHit u = sorted[k];
            if (!init_hit_inside(u, it)) {
                if (lane == 0) atomicOr(&a.cnt->flags, kFlagBadInitHit);
                continue;
            }
            if (contained(u, saved, nsaved, lane)) continue;
            const int32_t q_off = tasks[k].q_off;
            const int32_t s_off = q_off + (u.s_start - u.q_start);
            const int4 rl = res[2 * k], rr = res[2 * k + 1];
            int32_t left = rl.x, al = rl.y, bl = rl.z, right = rr.x, ar = rr.y, br = rr.z;
            if (rl.w < 0) {
                left = xdrop_dp<true>(it.qres, it.sub, q_off + 1, s_off + 1, a.gap_open, a.gap_extend, a.xdrop, mat, Hb,
                                      Eb, &al, &bl, &cells);
            } else {
                cells += static_cast<unsigned long long>(rl.w);
            }
            if (rr.w < 0) {
                ar = br = 0;
                right = xdrop_dp<false>(it.qres + q_off, it.sub + s_off, it.qlen - q_off - 1, it.slen - s_off - 1,
                                        a.gap_open, a.gap_extend, a.xdrop, mat, Hb, Eb, &ar, &br, &cells);
            } else {
                cells += static_cast<unsigned long long>(rr.w);
            }
            ++n_ext;
            const int32_t score = left + right;
            if (score >= it.cutoff) {
                if (lane == 0) saved[nsaved] = make_hsp(it.wi.subject, score, q_off, s_off, al, bl, ar, br);
                ++nsaved;
            }
            __syncwarp();
        }
        publish(a, it, saved, nsaved, lane);
    }
    if (lane == 0) {
        atomicAdd(&a.cnt->dp_cells, cells);
        atomicAdd(&a.cnt->gapped_ext, n_ext);
    }
}

// ------------------------------------------------------------------------
// Hit-list selection (hitlist_size, max_target_seqs), for the queries whose
// kept subjects outnumber their limit. The ranking key orders subjects by
// the score of their best HSP, then by smaller OID; keys within a query are
// distinct, so the k-th largest key is exact and exactly k lists stay.

__device__ __forceinline__ unsigned long long rank_key(const GroupDesc &g) {
    return (static_cast<unsigned long long>(static_cast<uint32_t>(g.best) ^ 0x80000000u) << 32) |
           static_cast<unsigned long long>(0xffffffffu - g.oid);
}

// Lays each selecting query's keys out in its own segment.
__global__ void hitlist_scatter_kernel(const HitlistArgs a) {
    for (unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
         g < a.n_groups; g += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const GroupDesc d = a.groups[g];
        const uint32_t lo = a.seg_off[d.query], hi = a.seg_off[d.query + 1];
        if (hi == lo) continue;
        const uint32_t pos = lo + atomicAdd(&a.seg_fill[d.query], 1u);
        if (pos >= hi) continue;  // cannot happen: the segment holds the query's published lists
        a.keys[pos] = rank_key(d);
        a.idx[pos] = static_cast<uint32_t>(g);
    }
}

// One block per selecting query: an MSB-first radix select (8-bit digits)
// finds the limit-th largest key; lists below it are dropped.
__global__ void __launch_bounds__(256) hitlist_select_kernel(const HitlistArgs a) {
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long s_prefix;
    __shared__ uint32_t s_rank;
    const uint32_t q = a.sel_queries[blockIdx.x];
    const uint32_t lo = a.seg_off[q], hi = a.seg_off[q + 1];
    unsigned long long prefix = 0, mask = 0;
    uint32_t rank = static_cast<uint32_t>(a.limit[q]);  // 1 <= rank < hi - lo
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const unsigned long long k = a.keys[i];
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 0xffu], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t above = 0;
            int b = 255;
            for (; b > 0 && above + hist[b] < rank; --b) above += hist[b];
            s_prefix = prefix | (static_cast<unsigned long long>(b) << shift);
            s_rank = rank - above;
        }
        __syncthreads();
        prefix = s_prefix;
        rank = s_rank;
        mask |= 0xffull << shift;
    }
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
        if (a.keys[i] < prefix) a.groups[a.idx[i]].n = 0u;
}

}  // namespace

cudaError_t launch_hitlist(const HitlistArgs &a, uint32_t n_select, int n_sm, cudaStream_t st) {
    if (a.n_groups == 0 || n_select == 0) return cudaSuccess;
    const unsigned long long want = (a.n_groups + 255) / 256;
    const int blocks = static_cast<int>(std::min<unsigned long long>(want, static_cast<unsigned long long>(n_sm) * 8));
    hitlist_scatter_kernel<<<blocks, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hitlist_select_kernel<<<n_select, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gapped(const GappedArgs &a, int n_blocks, cudaStream_t st, int warps_per_block) {
    if (warps_per_block < 1 || warps_per_block > kGappedWarpsPerBlock) return cudaErrorInvalidValue;
    gapped_kernel<<<n_blocks, warps_per_block * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gapped_split(const GappedArgs &a, int n_blocks, int n_sm, cudaStream_t st) {
    constexpr size_t ring_bytes = sizeof(uint32_t) * kDpWarpsPerBlock * kDpRing * 32;
    // per device: the DP kernel's occupancy
    constexpr int kMaxDevices = 64;
    static std::once_flag once[kMaxDevices];
    static cudaError_t setup_of[kMaxDevices];
    static int per_sm_of[kMaxDevices];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::call_once(once[dev], [dev] {
        per_sm_of[dev] = 1;
        setup_of[dev] = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_of[dev], gapped_dp_kernel,
                                                                      kDpWarpsPerBlock * 32, ring_bytes);
    });
    if (setup_of[dev] != cudaSuccess) return setup_of[dev];
    gapped_prep_kernel<<<n_blocks, kGappedWarpsPerBlock * 32, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    gapped_dp_kernel<<<n_sm * std::max(per_sm_of[dev], 1), kDpWarpsPerBlock * 32, ring_bytes, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    gapped_finish_kernel<<<n_blocks, kGappedWarpsPerBlock * 32, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t gapped_occupancy(int *blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gapped_kernel,
                                                         kGappedWarpsPerBlock * 32, 0);
}

}  // namespace blaze
