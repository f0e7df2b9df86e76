// traceback.cu -- the traceback stage on GB300 (sm_103a): every HSP of a
// preliminary result is aligned again from its gapped start point with the
// final X-drop, keeping the path, and its identities, mismatches and gaps are
// counted from that path (the published gapped-BLAST traceback; in the
// reference this is NCBI's traceback stage after the preliminary search,
// BLAZE_ncbi/prelim_stage.cpp:1462-1498).
//
// One warp per HSP. The left and right X-drop DPs run row-parallel exactly as
// in the gapped stage; every computed cell also stores a direction byte in
// the warp's buffer (row by row over the band). Lane 0 then walks the path
// back from the best cell.
#include <cstdint>

#include "common.cuh"

namespace blaze {
namespace {

__device__ const int32_t g_blosum_tb[kAlphabet * kAlphabet] = {
#include "blosum62.inc"
};

constexpr unsigned kFull = 0xffffffffu;
// direction byte: bits 0-1 where H came from (diagonal, vertical gap E,
// horizontal gap F); the E handed down extends; the F handed right extends;
// the cell is dead
constexpr uint8_t kTbDiag = 0, kTbE = 1, kTbF = 2, kTbEExt = 4, kTbFExt = 8, kTbDead = 128;

struct DirRows {
    uint8_t *dir;
    int32_t *rows;  // first, end, offset per row
    unsigned long long cap;
    uint32_t row_cap;
    bool overflow;
};

// The gapped stage's row-parallel X-drop DP with each computed cell's
// direction recorded. The sources follow the sequential recurrence: H takes
// the diagonal unless the vertical gap is larger, and either unless the
// horizontal gap is larger; a gap state handed on extends unless opening from
// H is strictly larger. (Values of dead cells may differ from the sequential
// DP's; a path never passes through one.)
template <bool REV>
__device__ int32_t xdrop_dp_dirs(const uint8_t *__restrict__ A, const uint8_t *__restrict__ B, int32_t M,
                                 int32_t N, int32_t gap_open, int32_t gap_extend, int32_t xdrop, const int32_t *mat,
                                 int32_t *Hb, int32_t *Eb, int32_t *a_best, int32_t *b_best, DirRows &d,
                                 int32_t *rows_used, int32_t *cells) {
    const int lane = threadIdx.x & 31;
    const int32_t goe = gap_open + gap_extend, ge = gap_extend;
    if (xdrop < goe) xdrop = goe;
    *a_best = 0;
    *b_best = 0;
    *rows_used = 0;
    if (M <= 0 || N <= 0) return 0;
    if (static_cast<uint32_t>(M) + 1 > d.row_cap || static_cast<unsigned long long>(N) + 2 > d.cap) {
        d.overflow = true;
        return 0;
    }
    int32_t bsize = 1 + min(N, (xdrop - goe) / ge + 1);
    for (int32_t i = lane; i < bsize; i += 32) {
        const int32_t h = i == 0 ? 0 : -goe - (i - 1) * ge;
        Hb[i] = h;
        Eb[i] = h - goe;
        d.dir[i] = i == 0 ? kTbDiag : static_cast<uint8_t>(kTbF | kTbFExt);  // row 0: gap from the origin
    }
    if (lane == 0) {
        d.rows[0] = 0;
        d.rows[1] = bsize;
        d.rows[2] = 0;
    }
    unsigned long long at = static_cast<unsigned long long>(bsize);
    __syncwarp();
    int32_t best = 0, first = 0, ab = 0, bb = 0, a = 1;
    for (; a <= M; ++a) {
        if (at + static_cast<unsigned long long>(N + 2 - first) > d.cap) {
            d.overflow = true;
            break;
        }
        const int32_t *row = mat + kAlphabet * (REV ? A[M - a] : A[a]);
        const int32_t row_first = first;
        *cells += bsize - first;
        int32_t carry_p = kNeg, carry_best = best, carry_hold = kNeg;
        int32_t first_alive = -1, last_alive = -1, row_best = best, row_best_b = -1;
        for (int32_t c0 = first; c0 < bsize; c0 += 32) {
            const int32_t b = c0 + lane;
            const bool act = b < bsize;
            const int32_t hold = act ? Hb[b] : kNeg;
            const int32_t ein = act ? Eb[b] : kNeg;
            int32_t hprev = __shfl_up_sync(kFull, hold, 1);
            if (lane == 0) hprev = carry_hold;
            const int32_t diag = (act && b > first) ? hprev + row[REV ? B[N - b] : B[b]] : kNeg;
            const int32_t D = max(ein, diag);
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
            // the best so far in row-major order: only a segment whose largest
            // H beats the carried best needs the prefix maximum
            const int32_t hv = act ? H : INT32_MIN;
            const int32_t cm = __reduce_max_sync(kFull, hv);
            int32_t cur_best = carry_best;
            if (cm > carry_best) {
                int32_t inclh = hv;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int32_t x = __shfl_up_sync(kFull, inclh, o);
                    if (lane >= o) inclh = max(inclh, x);
                }
                int32_t exclh = __shfl_up_sync(kFull, inclh, 1);
                if (lane == 0) exclh = INT32_MIN;
                cur_best = max(carry_best, exclh);
                const unsigned mm = __ballot_sync(kFull, act && H == cm);
                row_best = cm;
                row_best_b = c0 + __ffs(mm) - 1;
                carry_best = cm;
            }
            const bool alive = act && (cur_best - H <= xdrop);
            const unsigned am = __ballot_sync(kFull, alive);
            if (am) {
                if (first_alive < 0) first_alive = c0 + __ffs(am) - 1;
                last_alive = c0 + 31 - __clz(am);
            }
            carry_hold = __shfl_sync(kFull, hold, 31);
            carry_p = max(carry_p, __shfl_sync(kFull, incl, 31));
            __syncwarp();
            if (act) {
                uint8_t dv = kTbDead;
                if (alive) {
                    dv = max(diag, ein) < G ? kTbF : (diag < ein ? kTbE : kTbDiag);
                    if (!(H - goe > ein - ge)) dv |= kTbEExt;
                    if (!(H - goe > G - ge)) dv |= kTbFExt;
                    Eb[b] = max(H - goe, ein - ge);
                    Hb[b] = H;
                } else if (first_alive >= 0 && b > first_alive) {
                    Hb[b] = kNeg;
                }
                d.dir[at + static_cast<unsigned long long>(b - row_first)] = dv;
            }
            __syncwarp();
        }
        int32_t row_end = bsize;
        if (first_alive < 0) {
            if (lane == 0) {
                d.rows[3 * a] = row_first;
                d.rows[3 * a + 1] = row_end;
                d.rows[3 * a + 2] = static_cast<int32_t>(at);
            }
            at += static_cast<unsigned long long>(row_end - row_first);
            ++a;
            break;
        }
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
                    d.dir[at + static_cast<unsigned long long>(bsize + t - row_first)] =
                        static_cast<uint8_t>(kTbF | kTbFExt);  // the row gap continues
                }
                bsize += n_ext;
            }
            row_end = bsize;
        }
        if (bsize <= N) {
            if (lane == 0) {
                Hb[bsize] = kNeg;
                Eb[bsize] = kNeg;
                d.dir[at + static_cast<unsigned long long>(bsize - row_first)] = kTbDead;  // sentinel column
            }
            ++bsize;
            row_end = bsize;
        }
        if (lane == 0) {
            d.rows[3 * a] = row_first;
            d.rows[3 * a + 1] = row_end;
            d.rows[3 * a + 2] = static_cast<int32_t>(at);
        }
        at += static_cast<unsigned long long>(row_end - row_first);
        __syncwarp();
    }
    *rows_used = a;
    *a_best = ab;
    *b_best = bb;
    __syncwarp();
    return best;
}

struct Walk {
    int32_t pairs, identities, positives, gaps, gap_opens;
    int last_move;
    bool ok;
};

__device__ __forceinline__ bool dir_at(const DirRows &d, int32_t rows, int32_t a, int32_t b, uint8_t *v) {
    if (a < 0 || a >= rows) return false;
    const int32_t f = d.rows[3 * a], e = d.rows[3 * a + 1];
    if (b < f || b >= e) return false;
    *v = d.dir[static_cast<unsigned long long>(d.rows[3 * a + 2]) + static_cast<unsigned long long>(b - f)];
    return true;
}

// Lane 0: the path from (a, b) back to the origin.
template <bool REV>
__device__ Walk walk_back(const DirRows &d, int32_t rows, const uint8_t *A, const uint8_t *B, int32_t M, int32_t N,
                          int32_t a, int32_t b, const int32_t *mat) {
    Walk w{0, 0, 0, 0, 0, -1, true};
    int state = 0, prev = -1;
    long long guard = 2ll * (M + N) + 8;
    while ((a > 0 || b > 0) && guard-- > 0) {
        int move;
        uint8_t v = 0;
        if (state == 0) {
            if (a == 0) {
                state = 2;
                continue;
            }
            if (!dir_at(d, rows, a, b, &v) || (v & kTbDead)) {
                w.ok = false;
                return w;
            }
            const int src = v & 3;
            if (src == kTbDiag) {
                const uint32_t x = REV ? A[M - a] : A[a], y = REV ? B[N - b] : B[b];
                ++w.pairs;
                w.identities += x == y;
                w.positives += mat[x * kAlphabet + y] > 0;
                move = 0;
                --a;
                --b;
            } else {
                state = src == kTbE ? 1 : 2;
                continue;
            }
        } else if (state == 1) {
            if (a - 1 > 0 && !dir_at(d, rows, a - 1, b, &v)) {
                w.ok = false;
                return w;
            }
            move = 1;
            ++w.gaps;
            if (a - 1 == 0 || !(v & kTbEExt)) state = 0;
            --a;
        } else {
            if (!dir_at(d, rows, a, b - 1, &v)) {
                w.ok = false;
                return w;
            }
            move = 2;
            ++w.gaps;
            if (!(v & kTbFExt) || (a == 0 && b - 1 == 0)) state = 0;
            --b;
        }
        if (move != 0 && move != prev) ++w.gap_opens;
        prev = move;
        w.last_move = move;
    }
    w.ok = w.ok && a == 0 && b == 0;
    return w;
}

__global__ void __launch_bounds__(kTracebackWarpsPerBlock * 32) traceback_kernel(const TracebackArgs a) {
    __shared__ int32_t mat[kAlphabet * kAlphabet];
    for (int i = threadIdx.x; i < kAlphabet * kAlphabet; i += blockDim.x) mat[i] = g_blosum_tb[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned long long gwarp = (static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int32_t *Hb = a.dp + gwarp * 2ull * a.dp_stride;
    int32_t *Eb = Hb + a.dp_stride;
    DirRows d;
    d.dir = a.dirs + gwarp * a.dir_cap;
    d.rows = a.rows + gwarp * 3ull * a.row_cap;
    d.cap = a.dir_cap;
    d.row_cap = a.row_cap;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(a.cursor, 1ull);
        t = __shfl_sync(kFull, t, 0);
        if (t >= a.n_items) break;
        const TbItem it = a.items[t];
        const uint64_t o0 = a.off[it.subject];
        const uint8_t *sub = a.res + o0;
        const int32_t slen = static_cast<int32_t>(a.off[it.subject + 1] - o0);
        const int32_t q_off = it.q_off, s_off = it.s_off;
        const uint8_t *qres = a.batch_q ? a.batch_q[it.query] : a.q;
        const int32_t qlen = a.batch_q ? a.batch_qlen[it.query] : a.qlen;
        d.overflow = false;
        int32_t al, bl, ar = 0, br = 0, right = 0, rows, cells = 0;
        TbOut o{};
        const int32_t left = xdrop_dp_dirs<true>(qres, sub, q_off + 1, s_off + 1, a.gap_open, a.gap_extend, a.xdrop,
                                                 mat, Hb, Eb, &al, &bl, d, &rows, &cells);
        Walk wl{0, 0, 0, 0, 0, -1, true}, wr{0, 0, 0, 0, 0, -1, true};
        if (!d.overflow && lane == 0) wl = walk_back<true>(d, rows, qres, sub, q_off + 1, s_off + 1, al, bl, mat);
        __syncwarp();
        if (!d.overflow && q_off < qlen - 1 && s_off < slen - 1) {
            right = xdrop_dp_dirs<false>(qres + q_off, sub + s_off, qlen - q_off - 1, slen - s_off - 1, a.gap_open,
                                         a.gap_extend, a.xdrop, mat, Hb, Eb, &ar, &br, d, &rows, &cells);
            if (!d.overflow && lane == 0)
                wr = walk_back<false>(d, rows, qres + q_off, sub + s_off, qlen - q_off - 1, slen - s_off - 1, ar,
                                      br, mat);
        }
        if (lane == 0) {
            o.score = left + right;
            o.q_start = q_off + 1 - al;
            o.q_end = q_off + ar + 1;
            o.s_start = s_off + 1 - bl;
            o.s_end = s_off + br + 1;
            o.identities = wl.identities + wr.identities;
            o.positives = wl.positives + wr.positives;
            o.gaps = wl.gaps + wr.gaps;
            o.length = wl.pairs + wr.pairs + o.gaps;
            o.mismatches = wl.pairs + wr.pairs - o.identities;
            o.gap_opens = wl.gap_opens + wr.gap_opens - ((wl.last_move > 0 && wl.last_move == wr.last_move) ? 1 : 0);
            o.status = d.overflow ? 1 : ((wl.ok && wr.ok) ? 0 : 2);
            o.cells = cells;
            a.out[t] = o;
        }
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_traceback(const TracebackArgs &a, int n_blocks, cudaStream_t st) {
    traceback_kernel<<<n_blocks, kTracebackWarpsPerBlock * 32, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace blaze
