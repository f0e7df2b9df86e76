/* A C99 client of blaze_db_create_from_source: a BlastSeqSrc-shaped source
 * over an in-memory database (what an NCBI engine's adapter passes), checked
 * against blaze_db_create on the same residues.
 *
 *   seqsrc_client          no GPU expected: the call must report
 *                          BLAZE_ERR_NO_DEVICE ("status 3")
 *   seqsrc_client gpu      builds both databases, searches one query through
 *                          blaze_prelim_search on each and compares every
 *                          HSP byte for byte; then an iterator that skips odd
 *                          OIDs, and malformed sources that must be refused */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "blaze_prelim.h"

#define N_SUBJ 3000u
#define QLEN 300

static uint32_t rng_state = 12345u;
static uint32_t next_rand(void) {
    rng_state = rng_state * 1664525u + 1013904223u;
    return rng_state >> 8;
}
/* the 20 standard residues in NCBIstdaa codes */
static const uint8_t kStd[20] = {1, 16, 13, 4, 3, 15, 5, 7, 8, 9, 11, 10, 12, 6, 14, 17, 18, 20, 22, 19};

typedef struct {
    const uint8_t *res;
    const uint64_t *off;
    uint32_t n;
    int skip_odd;      /* iterator over even OIDs only */
    uint32_t iter_pos;
    int bad_code_oid;  /* >= 0: this OID's residues carry a 0 */
    int repeat_iter;   /* iterator returns OID 0 twice */
    int64_t tot_bias;  /* added to get_tot_len */
    int fetched, released;
    uint8_t scratch[4096];
} Source;

static int64_t get_num_seqs(void *u) { return ((Source *)u)->n; }
static int64_t get_seq_len(void *u, uint32_t oid) {
    Source *s = (Source *)u;
    return (int64_t)(s->off[oid + 1] - s->off[oid]);
}
static int get_sequence(void *u, uint32_t oid, const uint8_t **res, uint32_t *len) {
    Source *s = (Source *)u;
    if (oid >= s->n) return 1;
    *len = (uint32_t)(s->off[oid + 1] - s->off[oid]);
    *res = s->res + s->off[oid];
    if ((int)oid == s->bad_code_oid && *len > 0) {
        memcpy(s->scratch, *res, *len);
        s->scratch[*len / 2] = 0;
        *res = s->scratch;
    }
    s->fetched++;
    return 0;
}
static void release_sequence(void *u, uint32_t oid) {
    (void)oid;
    ((Source *)u)->released++;
}
static int64_t get_tot_len(void *u) {
    Source *s = (Source *)u;
    return (int64_t)s->off[s->n] + s->tot_bias;
}
static int64_t get_max_seq_len(void *u) {
    Source *s = (Source *)u;
    uint64_t m = 0;
    for (uint32_t i = 0; i < s->n; ++i)
        if (s->off[i + 1] - s->off[i] > m) m = s->off[i + 1] - s->off[i];
    return (int64_t)m;
}
static int64_t iter_next(void *u) {
    Source *s = (Source *)u;
    if (s->repeat_iter && s->iter_pos == 1) {
        s->iter_pos++;
        return 0;
    }
    while (s->iter_pos < s->n) {
        uint32_t o = s->iter_pos++;
        if (!s->skip_odd || o % 2 == 0) return o;
    }
    return -1;
}

static blaze_seq_source make_source(Source *s, int with_iter) {
    blaze_seq_source src;
    memset(&src, 0, sizeof src);
    src.user = s;
    src.get_num_seqs = get_num_seqs;
    src.get_sequence = get_sequence;
    src.release_sequence = release_sequence;
    src.get_seq_len = get_seq_len;
    src.get_tot_len = get_tot_len;
    src.get_max_seq_len = get_max_seq_len;
    src.iter_next = with_iter ? iter_next : NULL;
    return src;
}

static int search(blaze_db *db, const uint8_t *q, const blaze_params *p, blaze_hsp *out, uint64_t cap,
                  uint64_t *n) {
    blaze_search *s = NULL;
    int rc = blaze_search_create(db, &s);
    if (rc == BLAZE_OK) rc = blaze_prelim_search(s, q, QLEN, p, out, cap, n);
    blaze_search_free(s);
    return rc;
}

int main(int argc, char **argv) {
    int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
    static uint64_t off[N_SUBJ + 1];
    uint8_t q[QLEN];
    for (int i = 0; i < QLEN; ++i) q[i] = kStd[next_rand() % 20];
    off[0] = 0;
    for (uint32_t i = 0; i < N_SUBJ; ++i) off[i + 1] = off[i] + 30 + next_rand() % 800;
    uint8_t *res = (uint8_t *)malloc(off[N_SUBJ]);
    if (!res) return 2;
    for (uint64_t i = 0; i < off[N_SUBJ]; ++i) res[i] = kStd[next_rand() % 20];
    /* every 7th subject carries a query window with a few substitutions */
    for (uint32_t i = 0; i < N_SUBJ; i += 7) {
        uint32_t L = (uint32_t)(off[i + 1] - off[i]), w = L < 120 ? L : 120, qs = next_rand() % (QLEN - 120);
        for (uint32_t k = 0; k < w; ++k)
            res[off[i] + k] = (next_rand() % 3 == 0) ? kStd[next_rand() % 20] : q[qs + k];
    }
    Source S;
    memset(&S, 0, sizeof S);
    S.res = res;
    S.off = off;
    S.n = N_SUBJ;
    S.bad_code_oid = -1;
    blaze_seq_source src = make_source(&S, 0);
    blaze_db *db_src = NULL;
    int rc = blaze_db_create_from_source(0, &src, &db_src);
    if (!gpu) {
        printf("status %d\n", rc);
        free(res);
        return rc == BLAZE_ERR_NO_DEVICE ? 0 : 1;
    }
    if (rc != BLAZE_OK) {
        printf("from_source failed %d\n", rc);
        return 1;
    }
    if (S.fetched != (int)N_SUBJ || S.released != S.fetched) {
        printf("fetch/release %d %d\n", S.fetched, S.released);
        return 1;
    }
    blaze_db *db_flat = NULL;
    if ((rc = blaze_db_create(0, res, off, N_SUBJ, &db_flat)) != BLAZE_OK) return 1;
    uint64_t tot_a = 0, tot_b = 0;
    uint32_t n_a = 0, n_b = 0, mx_a = 0, mx_b = 0;
    blaze_db_info(db_src, &tot_a, &n_a, &mx_a);
    blaze_db_info(db_flat, &tot_b, &n_b, &mx_b);
    if (tot_a != tot_b || n_a != n_b || mx_a != mx_b) {
        printf("info differs\n");
        return 1;
    }
    blaze_params p;
    if (blaze_params_default(QLEN, off[N_SUBJ], N_SUBJ, 10.0, &p) != BLAZE_OK) return 1;
    enum { CAP = 1 << 16 };
    static blaze_hsp a[CAP], b[CAP], c[CAP];
    uint64_t na = 0, nb = 0, nc = 0;
    if (search(db_src, q, &p, a, CAP, &na) != BLAZE_OK || search(db_flat, q, &p, b, CAP, &nb) != BLAZE_OK) {
        printf("search failed\n");
        return 1;
    }
    if (na != nb || memcmp(a, b, sizeof(blaze_hsp) * na) != 0 || na < 50) {
        printf("differ %llu %llu\n", (unsigned long long)na, (unsigned long long)nb);
        return 1;
    }
    /* an iterator over even OIDs: same HSPs on even OIDs, none on odd ones */
    Source E = S;
    E.skip_odd = 1;
    E.iter_pos = 0;
    blaze_seq_source src_e = make_source(&E, 1);
    blaze_db *db_even = NULL;
    if (blaze_db_create_from_source(0, &src_e, &db_even) != BLAZE_OK) return 1;
    if (search(db_even, q, &p, c, CAP, &nc) != BLAZE_OK) return 1;
    uint64_t k = 0;
    for (uint64_t i = 0; i < nb; ++i) {
        if (b[i].oid % 2) continue;
        if (k >= nc || memcmp(&b[i], &c[k], sizeof(blaze_hsp)) != 0) {
            printf("even differs at %llu\n", (unsigned long long)i);
            return 1;
        }
        ++k;
    }
    if (k != nc) return 1;
    /* malformed sources create nothing */
    blaze_db *bad = NULL;
    Source B = S;
    B.bad_code_oid = 17;
    blaze_seq_source src_b = make_source(&B, 0);
    int r1 = blaze_db_create_from_source(0, &src_b, &bad);
    Source R = S;
    R.repeat_iter = 1;
    R.iter_pos = 0;
    blaze_seq_source src_r = make_source(&R, 1);
    int r2 = blaze_db_create_from_source(0, &src_r, &bad);
    Source T = S;
    T.tot_bias = 1;
    blaze_seq_source src_t = make_source(&T, 0);
    int r3 = blaze_db_create_from_source(0, &src_t, &bad);
    if (r1 != BLAZE_ERR_INVALID_ARG || r2 != BLAZE_ERR_INVALID_ARG || r3 != BLAZE_ERR_INVALID_ARG || bad) {
        printf("malformed accepted %d %d %d\n", r1, r2, r3);
        return 1;
    }
    printf("same %llu %llu\n", (unsigned long long)na, (unsigned long long)nc);
    blaze_db_free(db_src);
    blaze_db_free(db_flat);
    blaze_db_free(db_even);
    free(res);
    return 0;
}
