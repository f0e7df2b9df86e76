/*
 * blaze_oracle.c -- sequential CPU restatement of the BLASTP preliminary
 * search stage. TEST INFRASTRUCTURE ONLY (see blaze_oracle.h for the rules and
 * for why parity with NCBI BLAST+ 2.13.0 is unpinned).
 *
 * Everything here is deliberately literal: one subject at a time, hits in
 * subject order, one diagonal state per true diagonal, the gapped DP row by
 * row. The GPU library must reproduce these results bit for bit.
 */
#include "blaze_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_NEG (INT32_MIN / 2) /* "minus infinity" of the gapped DP */

/* BLOSUM62 in NCBIstdaa order (-,A,B,C,D,E,F,G,H,I,K,L,M,N,P,Q,R,S,T,V,W,X,Y,Z,U,*,O,J);
 * the values are the published matrix as laid out in BLAZE_gpu/util.hpp:30-57.
 * Row/column 0 (the gap letter) never occurs in valid input. */
const int32_t ORC_BLOSUM62[ORC_ALPHABET][ORC_ALPHABET] = {
    {-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768,-32768},
    {-32768,4,-2,0,-2,-1,-2,0,-2,-1,-1,-1,-1,-2,-1,-1,-1,1,0,0,-3,-1,-2,-1,0,-4,-1,-1},
    {-32768,-2,4,-3,4,1,-3,-1,0,-3,0,-4,-3,4,-2,0,-1,0,-1,-3,-4,-1,-3,0,-3,-4,-1,-3},
    {-32768,0,-3,9,-3,-4,-2,-3,-3,-1,-3,-1,-1,-3,-3,-3,-3,-1,-1,-1,-2,-1,-2,-3,9,-4,-1,-1},
    {-32768,-2,4,-3,6,2,-3,-1,-1,-3,-1,-4,-3,1,-1,0,-2,0,-1,-3,-4,-1,-3,1,-3,-4,-1,-3},
    {-32768,-1,1,-4,2,5,-3,-2,0,-3,1,-3,-2,0,-1,2,0,0,-1,-2,-3,-1,-2,4,-4,-4,-1,-3},
    {-32768,-2,-3,-2,-3,-3,6,-3,-1,0,-3,0,0,-3,-4,-3,-3,-2,-2,-1,1,-1,3,-3,-2,-4,-1,0},
    {-32768,0,-1,-3,-1,-2,-3,6,-2,-4,-2,-4,-3,0,-2,-2,-2,0,-2,-3,-2,-1,-3,-2,-3,-4,-1,-4},
    {-32768,-2,0,-3,-1,0,-1,-2,8,-3,-1,-3,-2,1,-2,0,0,-1,-2,-3,-2,-1,2,0,-3,-4,-1,-3},
    {-32768,-1,-3,-1,-3,-3,0,-4,-3,4,-3,2,1,-3,-3,-3,-3,-2,-1,3,-3,-1,-1,-3,-1,-4,-1,3},
    {-32768,-1,0,-3,-1,1,-3,-2,-1,-3,5,-2,-1,0,-1,1,2,0,-1,-2,-3,-1,-2,1,-3,-4,-1,-3},
    {-32768,-1,-4,-1,-4,-3,0,-4,-3,2,-2,4,2,-3,-3,-2,-2,-2,-1,1,-2,-1,-1,-3,-1,-4,-1,3},
    {-32768,-1,-3,-1,-3,-2,0,-3,-2,1,-1,2,5,-2,-2,0,-1,-1,-1,1,-1,-1,-1,-1,-1,-4,-1,2},
    {-32768,-2,4,-3,1,0,-3,0,1,-3,0,-3,-2,6,-2,0,0,1,0,-3,-4,-1,-2,0,-3,-4,-1,-3},
    {-32768,-1,-2,-3,-1,-1,-4,-2,-2,-3,-1,-3,-2,-2,7,-1,-2,-1,-1,-2,-4,-1,-3,-1,-3,-4,-1,-3},
    {-32768,-1,0,-3,0,2,-3,-2,0,-3,1,-2,0,0,-1,5,1,0,-1,-2,-2,-1,-1,4,-3,-4,-1,-2},
    {-32768,-1,-1,-3,-2,0,-3,-2,0,-3,2,-2,-1,0,-2,1,5,-1,-1,-3,-3,-1,-2,0,-3,-4,-1,-2},
    {-32768,1,0,-1,0,0,-2,0,-1,-2,0,-2,-1,1,-1,0,-1,4,1,-2,-3,-1,-2,0,-1,-4,-1,-2},
    {-32768,0,-1,-1,-1,-1,-2,-2,-2,-1,-1,-1,-1,0,-1,-1,-1,1,5,0,-2,-1,-2,-1,-1,-4,-1,-1},
    {-32768,0,-3,-1,-3,-2,-1,-3,-3,3,-2,1,1,-3,-2,-2,-3,-2,0,4,-3,-1,-1,-2,-1,-4,-1,2},
    {-32768,-3,-4,-2,-4,-3,1,-2,-2,-3,-3,-2,-1,-4,-4,-2,-3,-3,-2,-3,11,-1,2,-2,-2,-4,-1,-2},
    {-32768,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-4,-1,-1},
    {-32768,-2,-3,-2,-3,-2,3,-3,2,-1,-2,-1,-1,-2,-3,-1,-2,-2,-2,-1,2,-1,7,-2,-2,-4,-1,-1},
    {-32768,-1,0,-3,1,4,-3,-2,0,-3,1,-3,-1,0,-1,4,0,0,-1,-2,-2,-1,-2,4,-3,-4,-1,-3},
    {-32768,0,-3,9,-3,-4,-2,-3,-3,-1,-3,-1,-1,-3,-3,-3,-3,-1,-1,-1,-2,-1,-2,-3,9,-4,-1,-1},
    {-32768,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,-4,1,-4,-4},
    {-32768,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-1,-4,-1,-1},
    {-32768,-1,-3,-1,-3,-3,0,-4,-3,3,-3,3,2,-3,-3,-2,-2,-2,-1,2,-2,-1,-1,-3,-1,-4,-1,3}};

#define SC(a, b) (ORC_BLOSUM62[(a)][(b)])

static int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
static int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }

/* ------------------------------------------------------------------ lookup */

/* prelim_stage.cpp:135-155 enumerates every word whose score against the query
 * word reaches T, and prelim_stage.cpp:378-383 always keeps the query word
 * itself. Cells list query offsets in increasing order, the order in which the
 * query positions are indexed. */
static int word_is_neighbour(int w, int v, int32_t threshold) {
    if (v == w) return 1;
    int a = w / 784, b = (w / 28) % 28, c = w % 28;
    int x = v / 784, y = (v / 28) % 28, z = v % 28;
    return SC(a, x) + SC(b, y) + SC(c, z) >= threshold;
}

/* Neighbours of word w: every v with score(w, v) >= T, plus w itself, in
 * increasing word index. Enumerated letter by letter with a bound on the best
 * possible remaining score. Returns the count written to out (<= ORC_NWORDS). */
static int word_neighbours(int w, int32_t threshold, int32_t *out) {
    static int32_t row_max[ORC_ALPHABET];
    static int have_max = 0;
    if (!have_max) {
        for (int a = 0; a < ORC_ALPHABET; a++) {
            int32_t m = SC(a, 0);
            for (int b = 1; b < ORC_ALPHABET; b++) m = SC(a, b) > m ? SC(a, b) : m;
            row_max[a] = m;
        }
        have_max = 1;
    }
    int a = w / 784, b = (w / 28) % 28, c = w % 28, n = 0, self = 0;
    for (int x = 0; x < ORC_ALPHABET; x++) {
        int32_t s0 = SC(a, x);
        if (s0 + row_max[b] + row_max[c] < threshold && x != a) continue;
        for (int y = 0; y < ORC_ALPHABET; y++) {
            int32_t s1 = s0 + SC(b, y);
            if (s1 + row_max[c] < threshold && !(x == a && y == b)) continue;
            for (int z = 0; z < ORC_ALPHABET; z++) {
                int v = x * 784 + y * 28 + z;
                if (word_is_neighbour(w, v, threshold)) {
                    out[n++] = v;
                    self |= v == w;
                }
            }
        }
    }
    (void)self;
    return n;
}

int orc_lookup_build(const uint8_t *query, int32_t qlen, int32_t threshold, orc_lookup *out) {
    memset(out, 0, sizeof(*out));
    out->cell_start = (uint32_t *)calloc(ORC_NWORDS + 1, sizeof(uint32_t));
    if (!out->cell_start) return -1;
    int32_t nwords = qlen >= ORC_WORDSIZE ? qlen - ORC_WORDSIZE + 1 : 0;
    uint32_t *count = (uint32_t *)calloc(ORC_NWORDS, sizeof(uint32_t));
    int32_t *nb = (int32_t *)malloc(sizeof(int32_t) * ORC_NWORDS);
    int32_t *word_of = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nwords > 0 ? nwords : 1));
    if (!count || !word_of || !nb) { free(count); free(word_of); free(nb); return -1; }
    for (int32_t i = 0; i < nwords; i++) word_of[i] = query[i] * 784 + query[i + 1] * 28 + query[i + 2];
    for (int32_t i = 0; i < nwords; i++) {
        int k = word_neighbours(word_of[i], threshold, nb);
        for (int j = 0; j < k; j++) count[nb[j]]++;
    }
    uint32_t acc = 0;
    for (int v = 0; v < ORC_NWORDS; v++) { out->cell_start[v] = acc; acc += count[v]; }
    out->cell_start[ORC_NWORDS] = acc;
    out->n_offsets = acc;
    out->offsets = (uint32_t *)malloc(sizeof(uint32_t) * (acc ? acc : 1));
    if (!out->offsets) { free(count); free(word_of); free(nb); return -1; }
    memset(count, 0, sizeof(uint32_t) * ORC_NWORDS);
    for (int32_t i = 0; i < nwords; i++) {
        int k = word_neighbours(word_of[i], threshold, nb);
        for (int j = 0; j < k; j++) out->offsets[out->cell_start[nb[j]] + count[nb[j]]++] = (uint32_t)i;
    }
    free(count);
    free(word_of);
    free(nb);
    return 0;
}

void orc_lookup_free(orc_lookup *lk) {
    free(lk->cell_start);
    free(lk->offsets);
    memset(lk, 0, sizeof(*lk));
}

/* ------------------------------------------------------ ungapped extension */

/* Left X-drop extension ending at (s_off, q_off), inclusive, starting from
 * score 0; the walk visits s_off, s_off-1, ... and keeps the strictly best
 * prefix (gpuBLAZE.cu:679-777 is the warp-parallel form of the same walk). */
static int32_t extend_left(const uint8_t *q, const uint8_t *s, int32_t q_off, int32_t s_off,
                           int32_t xdrop, int32_t *length) {
    int32_t n = imin(s_off, q_off);
    int32_t best_i = n + 1, score = 0, maxscore = 0;
    for (int32_t i = n; i >= 0; i--) {
        score += SC(q[q_off - n + i], s[s_off - n + i]);
        if (score > maxscore) { maxscore = score; best_i = i; }
        if (maxscore - score >= xdrop) break;
    }
    *length = n - best_i + 1;
    return maxscore;
}

/* Right X-drop extension starting at (s_off, q_off) with running score
 * maxscore; stops when the score falls to <= 0 or drops by xdrop
 * (gpuBLAZE.cu:779-883). s_last_off is where the walk stopped. */
static int32_t extend_right(const uint8_t *q, int32_t qlen, const uint8_t *s, int32_t slen,
                            int32_t q_off, int32_t s_off, int32_t xdrop, int32_t maxscore,
                            int32_t *length, int32_t *s_last_off) {
    int32_t n = imin(slen - s_off, qlen - q_off);
    int32_t best_i = -1, score = maxscore, i;
    for (i = 0; i < n; i++) {
        score += SC(q[q_off + i], s[s_off + i]);
        if (score > maxscore) { maxscore = score; best_i = i; }
        if (score <= 0 || maxscore - score >= xdrop) break;
    }
    *length = best_i + 1;
    *s_last_off = s_off + i;
    return maxscore;
}

/* Two-hit ungapped extension from the second hit (q_off, s_off); s_left_off
 * is the end of the first hit. Right extension only runs when the left one
 * reached back to the first hit (gpuBLAZE.cu:1113-1148). */
static int32_t extend_two_hit(const uint8_t *q, int32_t qlen, const uint8_t *s, int32_t slen,
                              int32_t s_left_off, int32_t s_off, int32_t q_off, int32_t xdrop,
                              int32_t *hsp_q, int32_t *hsp_s, int32_t *hsp_len,
                              int32_t *right_extend, int32_t *s_last_off) {
    int32_t score = 0, left_score = 0, right_d = 0, left_d = 0, right_score = 0;
    for (int32_t i = 0; i < ORC_WORDSIZE; i++) {
        score += SC(q[q_off + i], s[s_off + i]);
        if (score > left_score) { left_score = score; right_d = i + 1; }
    }
    int32_t q_right = q_off + right_d, s_right = s_off + right_d;
    left_score = extend_left(q, s, q_right - 1, s_right - 1, xdrop, &left_d);
    right_d = 0;
    *right_extend = 0;
    *s_last_off = s_right;
    if (left_d >= s_right - s_left_off) {
        *right_extend = 1;
        right_score = extend_right(q, qlen, s, slen, q_right, s_right, xdrop, left_score, &right_d,
                                   s_last_off);
    }
    *hsp_q = q_right - left_d;
    *hsp_s = s_right - left_d;
    *hsp_len = left_d + right_d;
    return imax(left_score, right_score);
}

/* ------------------------------------------------------------ word finder */

typedef struct scratch {
    int32_t *last;   /* per true diagonal: subject offset of the last recorded hit */
    uint8_t *flag;   /* per true diagonal: an extension ran right on it */
    int32_t ndiag_cap;
    orc_init *inits;
    int32_t inits_cap;
    orc_hsp *hsps;
    int32_t hsps_cap;
    int32_t *dp;     /* 2 * (N + 2) for the gapped DP */
    int32_t dp_cap;
} scratch;

static int grow(void **p, int32_t *cap, int32_t need, size_t elem) {
    if (need <= *cap) return 0;
    int32_t nc = *cap ? *cap : 64;
    while (nc < need) nc *= 2;
    void *np = realloc(*p, (size_t)nc * elem);
    if (!np) return -1;
    *p = np;
    *cap = nc;
    return 0;
}

static void scratch_free(scratch *sc) {
    free(sc->last); free(sc->flag); free(sc->inits); free(sc->hsps); free(sc->dp);
    memset(sc, 0, sizeof(*sc));
}

static int cmp_init(const void *x, const void *y) {
    const orc_init *a = (const orc_init *)x, *b = (const orc_init *)y;
    if (a->score != b->score) return a->score > b->score ? -1 : 1;
    if (a->s_trig != b->s_trig) return a->s_trig < b->s_trig ? -1 : 1;
    if (a->q_trig != b->q_trig) return a->q_trig < b->q_trig ? -1 : 1;
    return 0;
}

/* Scan the subject's words in order; for each word, visit the query offsets
 * of its cell in increasing order; run the two-hit logic per diagonal. Init
 * hits are returned sorted by descending score, ties in discovery order
 * (subject offset, then query offset). */
static int32_t word_finder(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                           const uint8_t *subj, int32_t slen, uint32_t subject_index,
                           const orc_params *p, scratch *sc) {
    int32_t n = 0;
    if (slen < ORC_WORDSIZE || qlen < ORC_WORDSIZE) return 0;
    int32_t ndiag = qlen + slen;
    int32_t cap = sc->ndiag_cap;
    if (grow((void **)&sc->last, &cap, ndiag, sizeof(int32_t))) return -1;
    cap = sc->ndiag_cap;
    if (grow((void **)&sc->flag, &cap, ndiag, 1)) return -1;
    sc->ndiag_cap = cap;
    for (int32_t d = 0; d < ndiag; d++) { sc->last[d] = -p->window; sc->flag[d] = 0; }
    for (int32_t s = 0; s + ORC_WORDSIZE <= slen; s++) {
        int w = subj[s] * 784 + subj[s + 1] * 28 + subj[s + 2];
        for (uint32_t k = lk->cell_start[w]; k < lk->cell_start[w + 1]; k++) {
            int32_t q = (int32_t)lk->offsets[k];
            int32_t d = s - q + qlen - 1;
            if (sc->flag[d]) {
                if (s < sc->last[d]) continue; /* inside the last extension */
                sc->last[d] = s;
                sc->flag[d] = 0;
                continue;
            }
            int32_t diff = s - sc->last[d];
            if (diff >= p->window) { sc->last[d] = s; continue; }
            if (diff < ORC_WORDSIZE) continue;
            int32_t hq, hs, hl, rext, slast;
            int32_t score = extend_two_hit(query, qlen, subj, slen, sc->last[d] + ORC_WORDSIZE, s,
                                           q, p->ungapped_xdrop, &hq, &hs, &hl, &rext, &slast);
            if (score >= p->ungapped_cutoff) {
                if (grow((void **)&sc->inits, &sc->inits_cap, n + 1, sizeof(orc_init))) return -1;
                orc_init *h = &sc->inits[n++];
                h->subject = subject_index;
                h->q_start = hq; h->s_start = hs; h->len = hl; h->score = score;
                h->q_trig = q; h->s_trig = s;
            }
            if (rext) { sc->flag[d] = 1; sc->last[d] = slast - (ORC_WORDSIZE - 1); }
            else sc->last[d] = s;
        }
    }
    qsort(sc->inits, (size_t)n, sizeof(orc_init), cmp_init);
    return n;
}

/* ------------------------------------------------------------- gapped DP */

int32_t orc_gapped_start(const uint8_t *q, const uint8_t *s, int32_t q_start, int32_t s_start,
                         int32_t len) {
    /* gpuBLAZE.cu:1174-1208: centre of the best 11-residue window of the
     * ungapped HSP, or its first residue when no window scores above 0. */
    const int32_t win = 11;
    if (len <= win) return q_start + len / 2;
    int32_t score = 0;
    for (int32_t i = 0; i < win; i++) score += SC(q[q_start + i], s[s_start + i]);
    int32_t max_score = score, max_offset = q_start + win - 1;
    for (int32_t i = q_start + win; i < q_start + len; i++) {
        int32_t j = i - q_start + s_start;
        score -= SC(q[i - win], s[j - win]);
        score += SC(q[i], s[j]);
        if (score > max_score) { max_score = score; max_offset = i; }
    }
    if (max_score > 0) max_offset -= win / 2;
    else max_offset = q_start;
    return max_offset;
}

/* Score-only X-drop DP anchored at the origin. Rows are A letters, columns B
 * letters; cell (a,b) uses the a-th row letter and the b-th column letter.
 * The band of live columns [first, b_size) shrinks from the left while its
 * leading cells fail the X-drop test, is cut on the right after the last live
 * cell, or is extended along the row gap when the row ended live; one -inf
 * column closes it. Failing interior cells become -inf. This is the X-drop
 * form of gpuBLAZE.cu:356-677 with the band bookkeeping made exact. */
static int32_t semi_gapped(const uint8_t *A, const uint8_t *B, int32_t M, int32_t N, int32_t reverse,
                           int32_t gap_open, int32_t gap_extend, int32_t xdrop,
                           int32_t *a_best, int32_t *b_best, int32_t *work) {
    const int32_t goe = gap_open + gap_extend;
    if (xdrop < goe) xdrop = goe;
    *a_best = 0;
    *b_best = 0;
    if (M <= 0 || N <= 0) return 0;
    int32_t *Hb = work, *Eb = work + (N + 2);
    int32_t score = -goe, i;
    Hb[0] = 0;
    Eb[0] = -goe;
    for (i = 1; i <= N; i++) {
        if (score < -xdrop) break;
        Hb[i] = score;
        Eb[i] = score - goe;
        score -= gap_extend;
    }
    int32_t b_size = i, first = 0, best = 0;
    for (int32_t a = 1; a <= M; a++) {
        const int32_t *row = ORC_BLOSUM62[reverse ? A[M - a] : A[a]];
        int32_t h = ORC_NEG, f = ORC_NEG, last = first;
        for (int32_t b = first; b < b_size; b++) {
            int32_t e = Eb[b];
            int32_t next = ORC_NEG;
            if (b + 1 <= N) next = Hb[b] + row[reverse ? B[N - 1 - b] : B[b + 1]];
            if (h < e) h = e;
            if (h < f) h = f;
            if (best - h > xdrop) {
                if (b == first) first++;
                else Hb[b] = ORC_NEG;
            } else {
                last = b;
                if (h > best) { best = h; *a_best = a; *b_best = b; }
                f -= gap_extend;
                e -= gap_extend;
                Eb[b] = imax(h - goe, e);
                f = imax(h - goe, f);
                Hb[b] = h;
            }
            h = next;
        }
        if (first == b_size) break;
        if (last < b_size - 1) {
            b_size = last + 1;
        } else {
            while (f >= best - xdrop && b_size <= N) {
                Hb[b_size] = f;
                Eb[b_size] = f - goe;
                f -= gap_extend;
                b_size++;
            }
        }
        if (b_size <= N) {
            Hb[b_size] = ORC_NEG;
            Eb[b_size] = ORC_NEG;
            b_size++;
        }
    }
    return best;
}

int32_t orc_semi_gapped(const uint8_t *A, const uint8_t *B, int32_t M, int32_t N, int32_t reverse,
                        int32_t gap_open, int32_t gap_extend, int32_t xdrop, int32_t *a_best,
                        int32_t *b_best) {
    int32_t *work = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)((N > 0 ? N : 0) + 2));
    if (!work) return INT32_MIN;
    int32_t r = semi_gapped(A, B, M, N, reverse, gap_open, gap_extend, xdrop, a_best, b_best, work);
    free(work);
    return r;
}

/* ------------------------------------------------------------- traceback */

/* Direction byte of a DP cell: bits 0-1 where H came from (0 diagonal, 1
 * vertical gap E, 2 horizontal gap F), bit 2 the E passed down extends (else
 * it opens from H), bit 3 the F passed right extends (else it opens from H),
 * bit 7 the cell is dead (below the X-drop bound). */
enum { TB_DIAG = 0, TB_E = 1, TB_F = 2, TB_EEXT = 4, TB_FEXT = 8, TB_DEAD = 128 };

typedef struct tb_rows {
    int32_t *first, *end; /* per row a (0..rows): band [first, end) */
    int64_t *at;          /* per row: offset of column `first` in dir */
    uint8_t *dir;
    int64_t n_dir, cap_dir;
    int32_t rows;
} tb_rows;

static int tb_put(tb_rows *t, uint8_t v) {
    if (t->n_dir == t->cap_dir) {
        int64_t c = t->cap_dir ? 2 * t->cap_dir : 4096;
        uint8_t *p = (uint8_t *)realloc(t->dir, (size_t)c);
        if (!p) return -1;
        t->dir = p;
        t->cap_dir = c;
    }
    t->dir[t->n_dir++] = v;
    return 0;
}

/* The banded X-drop DP of semi_gapped with every computed cell's direction
 * kept (row 0 is the gap along the first row from the origin). */
static int32_t tb_dp(const uint8_t *A, const uint8_t *B, int32_t M, int32_t N, int32_t reverse,
                     int32_t gap_open, int32_t gap_extend, int32_t xdrop, int32_t *a_best, int32_t *b_best,
                     tb_rows *t) {
    const int32_t goe = gap_open + gap_extend;
    if (xdrop < goe) xdrop = goe;
    *a_best = 0;
    *b_best = 0;
    t->rows = 0;
    t->n_dir = 0;
    if (M <= 0 || N <= 0) return 0;
    int32_t *Hb = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N + 2));
    int32_t *Eb = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N + 2));
    t->first = (int32_t *)malloc(sizeof(int32_t) * (size_t)(M + 1));
    t->end = (int32_t *)malloc(sizeof(int32_t) * (size_t)(M + 1));
    t->at = (int64_t *)malloc(sizeof(int64_t) * (size_t)(M + 1));
    if (!Hb || !Eb || !t->first || !t->end || !t->at) {
        free(Hb);
        free(Eb);
        return INT32_MIN;
    }
    int32_t score = -goe, i;
    Hb[0] = 0;
    Eb[0] = -goe;
    t->first[0] = 0;
    t->at[0] = 0;
    tb_put(t, TB_DIAG); /* the origin */
    for (i = 1; i <= N; i++) {
        if (score < -xdrop) break;
        Hb[i] = score;
        Eb[i] = score - goe;
        score -= gap_extend;
        tb_put(t, (uint8_t)(TB_F | (i > 1 ? 0 : 0) | TB_FEXT)); /* along row 0 from the origin */
    }
    t->end[0] = i;
    t->rows = 1;
    int32_t b_size = i, first = 0, best = 0;
    for (int32_t a = 1; a <= M; a++) {
        const int32_t *row = ORC_BLOSUM62[reverse ? A[M - a] : A[a]];
        int32_t h = ORC_NEG, f = ORC_NEG, last = first;
        t->first[a] = first;
        t->at[a] = t->n_dir;
        for (int32_t b = first; b < b_size; b++) {
            const int32_t diag = h;
            int32_t e = Eb[b];
            int32_t next = ORC_NEG;
            if (b + 1 <= N) next = Hb[b] + row[reverse ? B[N - 1 - b] : B[b + 1]];
            uint8_t d = TB_DIAG;
            if (h < e) { h = e; d = TB_E; }
            if (h < f) { h = f; d = TB_F; }
            if (best - h > xdrop) {
                if (b == first) first++;
                else Hb[b] = ORC_NEG;
                d = TB_DEAD;
            } else {
                last = b;
                if (h > best) { best = h; *a_best = a; *b_best = b; }
                f -= gap_extend;
                e -= gap_extend;
                if (!(h - goe > e)) d |= TB_EEXT;
                if (!(h - goe > f)) d |= TB_FEXT;
                Eb[b] = imax(h - goe, e);
                f = imax(h - goe, f);
                Hb[b] = h;
            }
            (void)diag;
            tb_put(t, d);
            h = next;
        }
        int32_t row_end = b_size;
        if (first == b_size) {
            t->end[a] = row_end;
            t->rows = a + 1;
            break;
        }
        if (last < b_size - 1) {
            b_size = last + 1;
        } else {
            while (f >= best - xdrop && b_size <= N) {
                Hb[b_size] = f;
                Eb[b_size] = f - goe;
                f -= gap_extend;
                b_size++;
                tb_put(t, (uint8_t)(TB_F | TB_FEXT)); /* the row gap continues */
            }
            row_end = b_size;
        }
        if (b_size <= N) {
            Hb[b_size] = ORC_NEG;
            Eb[b_size] = ORC_NEG;
            b_size++;
            tb_put(t, TB_DEAD); /* sentinel column */
            row_end = b_size;
        }
        t->end[a] = row_end;
        t->rows = a + 1;
    }
    free(Hb);
    free(Eb);
    return best;
}

typedef struct tb_walk {
    int32_t pairs, identities, positives, gaps, gap_opens;
    int last_move; /* move next to the origin: 0 pair, 1 vertical gap, 2 horizontal gap */
    char *ops;     /* optional: moves from the best cell back to the origin */
    int32_t n_ops, cap_ops;
} tb_walk;

static uint8_t tb_at(const tb_rows *t, int32_t a, int32_t b, int *ok) {
    if (a < 0 || a >= t->rows || b < t->first[a] || b >= t->end[a]) {
        *ok = 0;
        return TB_DEAD;
    }
    return t->dir[t->at[a] + (b - t->first[a])];
}

/* Walks from (a, b) back to the origin; letters A[row], B[col] as in tb_dp. */
static int tb_walk_back(const tb_rows *t, const uint8_t *A, const uint8_t *B, int32_t M, int32_t N, int32_t reverse,
                        int32_t a, int32_t b, tb_walk *w) {
    char *ops = w->ops;
    const int32_t cap = w->cap_ops;
    memset(w, 0, sizeof(*w));
    w->ops = ops;
    w->cap_ops = cap;
    w->last_move = -1;
    int state = 0; /* 0 H, 1 E, 2 F */
    int prev_move = -1, ok = 1;
    int64_t guard = (int64_t)(M + 1) * (N + 1) + 8;
    while ((a > 0 || b > 0) && guard-- > 0) {
        int move;
        if (state == 0) {
            if (a == 0) { state = 2; continue; } /* row 0: gap from the origin */
            const uint8_t d = tb_at(t, a, b, &ok);
            if (!ok || (d & TB_DEAD)) return -1;
            const int src = d & 3;
            if (src == TB_DIAG) {
                const uint8_t x = reverse ? A[M - a] : A[a], y = reverse ? B[N - b] : B[b];
                w->pairs++;
                if (x == y) w->identities++;
                if (ORC_BLOSUM62[x][y] > 0) w->positives++;
                move = 0;
                a--;
                b--;
            } else {
                state = src == TB_E ? 1 : 2;
                continue;
            }
        } else if (state == 1) { /* E at (a, b): from the cell above */
            const uint8_t d = a - 1 == 0 ? 0 : tb_at(t, a - 1, b, &ok);
            if (!ok) return -1;
            move = 1;
            w->gaps++;
            if (a - 1 == 0 || !(d & TB_EEXT)) state = 0;
            a--;
        } else { /* F at (a, b): from the cell on the left */
            const uint8_t d = tb_at(t, a, b - 1, &ok);
            if (!ok) return -1;
            move = 2;
            w->gaps++;
            if (!(d & TB_FEXT) || (a == 0 && b - 1 == 0)) state = 0;
            b--;
        }
        if (move != 0 && move != prev_move) w->gap_opens++;
        prev_move = move;
        w->last_move = move;
        if (w->ops && w->n_ops < w->cap_ops) w->ops[w->n_ops++] = move == 0 ? 'M' : move == 1 ? 'I' : 'D';
    }
    return (a == 0 && b == 0) ? 0 : -1;
}

int orc_traceback_ops(const uint8_t *query, int32_t qlen, const uint8_t *subject, int32_t slen, int32_t q_off,
                      int32_t s_off, int32_t gap_open, int32_t gap_extend, int32_t xdrop, orc_tb *out, char *ops,
                      int32_t ops_cap, int32_t *n_ops) {
    memset(out, 0, sizeof(*out));
    tb_rows t;
    memset(&t, 0, sizeof(t));
    int32_t al, bl, ar = 0, br = 0, right = 0;
    tb_walk wl, wr;
    memset(&wl, 0, sizeof(wl));
    memset(&wr, 0, sizeof(wr));
    wr.last_move = -1;
    /* the left walk runs from the leftmost column: its moves are in order;
     * the right walk's moves are reversed into the tail */
    wl.ops = ops;
    wl.cap_ops = ops ? ops_cap : 0;
    char *rops = ops ? (char *)malloc((size_t)(ops_cap > 0 ? ops_cap : 1)) : NULL;
    wr.ops = rops;
    wr.cap_ops = rops ? ops_cap : 0;
    int32_t left = tb_dp(query, subject, q_off + 1, s_off + 1, 1, gap_open, gap_extend, xdrop, &al, &bl, &t);
    int rc = left == INT32_MIN ? -1 : tb_walk_back(&t, query, subject, q_off + 1, s_off + 1, 1, al, bl, &wl);
    if (rc == 0 && q_off < qlen - 1 && s_off < slen - 1) {
        free(t.first); free(t.end); free(t.at);
        t.first = NULL; t.end = NULL; t.at = NULL;
        right = tb_dp(query + q_off, subject + s_off, qlen - q_off - 1, slen - s_off - 1, 0, gap_open, gap_extend,
                      xdrop, &ar, &br, &t);
        rc = right == INT32_MIN ? -1 : tb_walk_back(&t, query + q_off, subject + s_off, qlen - q_off - 1,
                                                    slen - s_off - 1, 0, ar, br, &wr);
    }
    free(t.first); free(t.end); free(t.at); free(t.dir);
    if (ops && n_ops) {
        int32_t n = wl.n_ops;
        for (int32_t k = wr.n_ops - 1; k >= 0 && n < ops_cap; k--) ops[n++] = rops[k];
        *n_ops = n;
    }
    free(rops);
    if (rc != 0) return -1;
    out->score = left + right;
    out->q_start = q_off + 1 - al;
    out->q_end = q_off + ar + 1;
    out->s_start = s_off + 1 - bl;
    out->s_end = s_off + br + 1;
    out->identities = wl.identities + wr.identities;
    out->positives = wl.positives + wr.positives;
    out->gaps = wl.gaps + wr.gaps;
    out->length = wl.pairs + wr.pairs + out->gaps;
    out->mismatches = wl.pairs + wr.pairs - out->identities;
    out->gap_opens = wl.gap_opens + wr.gap_opens;
    /* one gap run across the start point is one opening */
    if (wl.last_move > 0 && wl.last_move == wr.last_move) out->gap_opens--;
    return 0;
}

int orc_traceback(const uint8_t *query, int32_t qlen, const uint8_t *subject, int32_t slen, int32_t q_off,
                  int32_t s_off, int32_t gap_open, int32_t gap_extend, int32_t xdrop, orc_tb *out) {
    return orc_traceback_ops(query, qlen, subject, slen, q_off, s_off, gap_open, gap_extend, xdrop, out, NULL, 0,
                             NULL);
}

/* --------------------------------------------------- purge and final sort */

static int cmp_start(const void *x, const void *y) {
    const orc_hsp *a = (const orc_hsp *)x, *b = (const orc_hsp *)y;
    if (a->q_start != b->q_start) return a->q_start < b->q_start ? -1 : 1;
    if (a->s_start != b->s_start) return a->s_start < b->s_start ? -1 : 1;
    if (a->score != b->score) return a->score > b->score ? -1 : 1;
    if (a->q_end != b->q_end) return a->q_end > b->q_end ? -1 : 1;
    if (a->s_end != b->s_end) return a->s_end > b->s_end ? -1 : 1;
    return 0;
}

static int cmp_end(const void *x, const void *y) {
    const orc_hsp *a = (const orc_hsp *)x, *b = (const orc_hsp *)y;
    if (a->q_end != b->q_end) return a->q_end < b->q_end ? -1 : 1;
    if (a->s_end != b->s_end) return a->s_end < b->s_end ? -1 : 1;
    if (a->score != b->score) return a->score > b->score ? -1 : 1;
    if (a->q_start != b->q_start) return a->q_start < b->q_start ? -1 : 1;
    if (a->s_start != b->s_start) return a->s_start < b->s_start ? -1 : 1;
    return 0;
}

static int cmp_score(const void *x, const void *y) {
    const orc_hsp *a = (const orc_hsp *)x, *b = (const orc_hsp *)y;
    if (a->score != b->score) return a->score > b->score ? -1 : 1;
    if (a->s_start != b->s_start) return a->s_start < b->s_start ? -1 : 1;
    if (a->s_end != b->s_end) return a->s_end > b->s_end ? -1 : 1;
    if (a->q_start != b->q_start) return a->q_start < b->q_start ? -1 : 1;
    if (a->q_end != b->q_end) return a->q_end > b->q_end ? -1 : 1;
    return 0;
}

/* Drop HSPs that share their start point, then their end point, with a
 * better one; then order by score (blast_engine.c:792 and :801 call sites). */
static int32_t purge_and_sort(orc_hsp *h, int32_t n) {
    if (n <= 1) return n;
    qsort(h, (size_t)n, sizeof(orc_hsp), cmp_start);
    int32_t m = 0;
    for (int32_t i = 0; i < n; i++)
        if (m == 0 || h[i].q_start != h[m - 1].q_start || h[i].s_start != h[m - 1].s_start) h[m++] = h[i];
    n = m;
    qsort(h, (size_t)n, sizeof(orc_hsp), cmp_end);
    m = 0;
    for (int32_t i = 0; i < n; i++)
        if (m == 0 || h[i].q_end != h[m - 1].q_end || h[i].s_end != h[m - 1].s_end) h[m++] = h[i];
    n = m;
    qsort(h, (size_t)n, sizeof(orc_hsp), cmp_score);
    return n;
}

/* --------------------------------------------------------- gapped stage */

static int32_t gapped_stage(const uint8_t *query, int32_t qlen, const uint8_t *subj, int32_t slen,
                            uint32_t subject_index, const orc_params *p, const orc_init *inits,
                            int32_t n_inits, scratch *sc) {
    int32_t nh = 0;
    if (grow((void **)&sc->dp, &sc->dp_cap, 2 * (imax(qlen, slen) + 2), sizeof(int32_t))) return -1;
    for (int32_t k = 0; k < n_inits; k++) {
        const orc_init *u = &inits[k];
        /* skip an ungapped HSP that lies inside an already kept gapped HSP
         * scoring at least as much */
        int contained = 0;
        for (int32_t j = 0; j < nh && !contained; j++) {
            const orc_hsp *g = &sc->hsps[j];
            if (u->score <= g->score && g->q_start <= u->q_start && u->q_start + u->len <= g->q_end &&
                g->s_start <= u->s_start && u->s_start + u->len <= g->s_end)
                contained = 1;
        }
        if (contained) continue;
        int32_t q_off = orc_gapped_start(query, subj, u->q_start, u->s_start, u->len);
        int32_t s_off = q_off + (u->s_start - u->q_start);
        int32_t al, bl, ar = 0, br = 0, right = 0;
        int32_t left = semi_gapped(query, subj, q_off + 1, s_off + 1, 1, p->gap_open, p->gap_extend,
                                   p->gapped_xdrop, &al, &bl, sc->dp);
        if (q_off < qlen - 1 && s_off < slen - 1)
            right = semi_gapped(query + q_off, subj + s_off, qlen - q_off - 1, slen - s_off - 1, 0,
                                p->gap_open, p->gap_extend, p->gapped_xdrop, &ar, &br, sc->dp);
        int32_t score = left + right;
        if (score < p->gapped_cutoff) continue;
        if (grow((void **)&sc->hsps, &sc->hsps_cap, nh + 1, sizeof(orc_hsp))) return -1;
        orc_hsp *g = &sc->hsps[nh++];
        g->subject = subject_index;
        g->score = score;
        g->q_start = q_off + 1 - al;
        g->q_end = q_off + ar + 1;
        g->s_start = s_off + 1 - bl;
        g->s_end = s_off + br + 1;
        g->q_gstart = q_off;
        g->s_gstart = s_off;
    }
    return purge_and_sort(sc->hsps, nh);
}

static int32_t subject_hsps(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                            const uint8_t *subj, int32_t slen, uint32_t subject_index,
                            const orc_params *p, scratch *sc) {
    int32_t ni = word_finder(query, qlen, lk, subj, slen, subject_index, p, sc);
    if (ni <= 0) return ni;
    return gapped_stage(query, qlen, subj, slen, subject_index, p, sc->inits, ni, sc);
}

int32_t orc_subject_inits(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                          const uint8_t *subj, int32_t slen, uint32_t subject_index,
                          const orc_params *p, orc_init *out, int32_t cap) {
    scratch sc;
    memset(&sc, 0, sizeof(sc));
    int32_t n = word_finder(query, qlen, lk, subj, slen, subject_index, p, &sc);
    for (int32_t i = 0; i < n && i < cap; i++) out[i] = sc.inits[i];
    scratch_free(&sc);
    return n;
}

int32_t orc_subject_hsps(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                         const uint8_t *subj, int32_t slen, uint32_t subject_index,
                         const orc_params *p, orc_hsp *out, int32_t cap) {
    scratch sc;
    memset(&sc, 0, sizeof(sc));
    int32_t n = subject_hsps(query, qlen, lk, subj, slen, subject_index, p, &sc);
    for (int32_t i = 0; i < n && i < cap; i++) out[i] = sc.hsps[i];
    scratch_free(&sc);
    return n;
}

/* ------------------------------------------------------- whole database */

#define ORC_CHUNK 256

typedef struct chunk_out {
    orc_hsp *hsps;
    int32_t n_hsps;
    orc_init *inits;
    int32_t n_inits;
} chunk_out;

struct orc_result {
    uint64_t n_hsps, n_inits;
    orc_hsp *hsps;
    orc_init *inits;
};

typedef struct job {
    const uint8_t *query;
    int32_t qlen;
    const orc_lookup *lk;
    const uint8_t *residues;
    const uint64_t *offsets;
    uint32_t n_subjects;
    const orc_params *p;
    int32_t want_inits;
    uint32_t n_chunks;
    chunk_out *chunks;
    uint32_t next; /* guarded by lock */
    pthread_mutex_t lock;
    int failed;
} job;

static int append(void **arr, int32_t *n, int32_t *cap, const void *src, int32_t k, size_t elem) {
    if (grow(arr, cap, *n + k, elem)) return -1;
    memcpy((char *)*arr + (size_t)*n * elem, src, (size_t)k * elem);
    *n += k;
    return 0;
}

static void *worker(void *arg) {
    job *jb = (job *)arg;
    scratch sc;
    memset(&sc, 0, sizeof(sc));
    for (;;) {
        pthread_mutex_lock(&jb->lock);
        uint32_t c = jb->next++;
        pthread_mutex_unlock(&jb->lock);
        if (c >= jb->n_chunks) break;
        chunk_out *co = &jb->chunks[c];
        int32_t hcap = 0, icap = 0;
        uint32_t lo = c * ORC_CHUNK, hi = lo + ORC_CHUNK;
        if (hi > jb->n_subjects) hi = jb->n_subjects;
        for (uint32_t i = lo; i < hi; i++) {
            const uint8_t *subj = jb->residues + jb->offsets[i];
            int32_t slen = (int32_t)(jb->offsets[i + 1] - jb->offsets[i]);
            int32_t ni = word_finder(jb->query, jb->qlen, jb->lk, subj, slen, i, jb->p, &sc);
            if (ni < 0) { jb->failed = 1; break; }
            if (ni == 0) continue;
            if (jb->want_inits &&
                append((void **)&co->inits, &co->n_inits, &icap, sc.inits, ni, sizeof(orc_init))) {
                jb->failed = 1;
                break;
            }
            int32_t nh = gapped_stage(jb->query, jb->qlen, subj, slen, i, jb->p, sc.inits, ni, &sc);
            if (nh < 0) { jb->failed = 1; break; }
            if (nh && append((void **)&co->hsps, &co->n_hsps, &hcap, sc.hsps, nh, sizeof(orc_hsp))) {
                jb->failed = 1;
                break;
            }
        }
    }
    scratch_free(&sc);
    return NULL;
}

orc_result *orc_search_db(const uint8_t *query, int32_t qlen, const uint8_t *residues,
                          const uint64_t *offsets, uint32_t n_subjects, const orc_params *p,
                          int32_t n_threads, int32_t want_inits) {
    orc_lookup lk;
    if (orc_lookup_build(query, qlen, p->word_threshold, &lk)) return NULL;
    job jb;
    memset(&jb, 0, sizeof(jb));
    jb.query = query; jb.qlen = qlen; jb.lk = &lk; jb.residues = residues; jb.offsets = offsets;
    jb.n_subjects = n_subjects; jb.p = p; jb.want_inits = want_inits;
    jb.n_chunks = (n_subjects + ORC_CHUNK - 1) / ORC_CHUNK;
    jb.chunks = (chunk_out *)calloc(jb.n_chunks ? jb.n_chunks : 1, sizeof(chunk_out));
    pthread_mutex_init(&jb.lock, NULL);
    if (n_threads < 1) n_threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    for (int32_t t = 0; t < n_threads; t++) pthread_create(&th[t], NULL, worker, &jb);
    for (int32_t t = 0; t < n_threads; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&jb.lock);
    orc_lookup_free(&lk);
    orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
    for (uint32_t c = 0; c < jb.n_chunks; c++) {
        r->n_hsps += (uint64_t)jb.chunks[c].n_hsps;
        r->n_inits += (uint64_t)jb.chunks[c].n_inits;
    }
    r->hsps = (orc_hsp *)malloc(sizeof(orc_hsp) * (r->n_hsps ? r->n_hsps : 1));
    r->inits = (orc_init *)malloc(sizeof(orc_init) * (r->n_inits ? r->n_inits : 1));
    uint64_t h = 0, k = 0;
    for (uint32_t c = 0; c < jb.n_chunks; c++) {
        chunk_out *co = &jb.chunks[c];
        if (co->n_hsps) memcpy(r->hsps + h, co->hsps, sizeof(orc_hsp) * (size_t)co->n_hsps);
        if (co->n_inits) memcpy(r->inits + k, co->inits, sizeof(orc_init) * (size_t)co->n_inits);
        h += (uint64_t)co->n_hsps;
        k += (uint64_t)co->n_inits;
        free(co->hsps);
        free(co->inits);
    }
    free(jb.chunks);
    if (jb.failed) { orc_result_free(r); return NULL; }
    return r;
}

uint64_t orc_result_n_hsps(const orc_result *r) { return r->n_hsps; }
uint64_t orc_result_n_inits(const orc_result *r) { return r->n_inits; }
void orc_result_copy_hsps(const orc_result *r, orc_hsp *out) {
    if (r->n_hsps) memcpy(out, r->hsps, sizeof(orc_hsp) * r->n_hsps);
}
void orc_result_copy_inits(const orc_result *r, orc_init *out) {
    if (r->n_inits) memcpy(out, r->inits, sizeof(orc_init) * r->n_inits);
}
void orc_result_free(orc_result *r) {
    if (!r) return;
    free(r->hsps);
    free(r->inits);
    free(r);
}

/* ------------------------------------------------------ Karlin-Altschul */

double orc_evalue(int32_t score, double lambda, double K, double searchsp) {
    return searchsp * K * exp(-lambda * (double)score);
}

/* Largest integer ell >= 0 below the fixed point of
 *   f(ell) = beta + (alpha/lambda) * (ln K + ln((m - ell) * (n - N*ell)))
 * that keeps K*(m-ell)*(n-N*ell) above max(m, n) (Altschul & Gish edge
 * correction, as used for BLAST effective lengths). */
int32_t orc_length_adjustment(double K, double logK, double alpha_d_lambda, double beta,
                              int32_t query_length, int64_t db_length, int64_t db_num_seqs) {
    double m = (double)query_length, n = (double)db_length, N = (double)db_num_seqs;
    double floor_sp = m > n ? m : n;
    int32_t lo = 0, hi = query_length > 0 ? query_length - 1 : 0;
    int32_t best = 0;
    while (lo <= hi) {
        int32_t ell = lo + (hi - lo) / 2;
        double mm = m - ell, nn = n - N * ell;
        int ok = mm > 0 && nn > 0 && K * mm * nn > floor_sp;
        if (ok) {
            double f = beta + alpha_d_lambda * (logK + log(mm) + log(nn));
            ok = f > (double)ell;
        }
        if (ok) { best = ell; lo = ell + 1; }
        else hi = ell - 1;
    }
    return best;
}
