/*
 * blaze_oracle.h -- CPU oracle for the BLASTP preliminary search stage.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load this library, and
 * only as the checker. The product (libblaze103) never links or calls it.
 *
 * PARITY UNPINNED against NCBI BLAST+ 2.13.0: the arithmetic of the stage
 * lives in un-vendored NCBI sources (aa_ungapped.c, blast_gapalign.c,
 * blast_hits.c, blast_stat.c of ncbi-blast-2.13.0+-src, downloaded by the
 * reference's build.sh:45-51) which are absent here, and the reference ships no
 * golden vectors. This file restates, in plain sequential C, the published
 * gapped-BLAST method (Altschul et al. 1997, NAR 25:3389) in the form the
 * reference's own code follows:
 *   - BLOSUM62 in NCBIstdaa order ............ BLAZE_gpu/util.hpp:30-57
 *   - neighbourhood words, exact word kept ... BLAZE_ncbi/prelim_stage.cpp:135-155, 360-386
 *   - two-hit diagonal logic, window 40 ...... BLAZE_gpu/gpuBLAZE.cu:1016-1049
 *   - ungapped X-drop left/right ............. BLAZE_gpu/gpuBLAZE.cu:679-883, 1096-1152
 *   - gapped start over an 11-window ......... BLAZE_gpu/gpuBLAZE.cu:1154-1215
 *   - score-only semi-gapped X-drop DP ....... BLAZE_gpu/gpuBLAZE.cu:356-677 (X-drop form)
 *   - per-subject pipeline order (word finder, gapped score, purge, sort,
 *     E-values, prelim reap) ................. BLAZE_ncbi/blast_engine.c:654-853, 896-932, 1423-1477
 * Where the reference leaves a choice to NCBI code, the function restating
 * it says which published rule it follows.
 */
#ifndef BLAZE_ORACLE_H
#define BLAZE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_ALPHABET 28
#define ORC_NWORDS (28 * 28 * 28)
#define ORC_WORDSIZE 3

typedef struct orc_params {
    int32_t word_threshold;  /* neighbourhood threshold T (11) */
    int32_t window;          /* two-hit window (40) */
    int32_t ungapped_xdrop;  /* raw ungapped X-drop (16) */
    int32_t ungapped_cutoff; /* raw score an ungapped HSP needs to be gapped-extended */
    int32_t gap_open;        /* 11 */
    int32_t gap_extend;      /* 1 */
    int32_t gapped_xdrop;    /* raw gapped X-drop of the preliminary stage (38) */
    int32_t gapped_cutoff;   /* raw score a gapped HSP needs to be kept */
} orc_params;

/* One gapped HSP. Offsets are 0-based, ends exclusive. */
typedef struct orc_hsp {
    uint32_t subject;  /* index of the subject in the searched array */
    int32_t score;
    int32_t q_start, q_end;
    int32_t s_start, s_end;
    int32_t q_gstart, s_gstart; /* start point of the gapped extension */
} orc_hsp;

/* One ungapped extension that reached the ungapped cutoff (an "init hit"). */
typedef struct orc_init {
    uint32_t subject;
    int32_t q_start, s_start, len, score;
    int32_t q_trig, s_trig; /* the second word hit that triggered it */
} orc_init;

/* Word lookup: cell w holds the query offsets (ascending) whose word scores
 * >= T against w, or equals w. */
typedef struct orc_lookup {
    uint32_t *cell_start; /* ORC_NWORDS + 1 prefix offsets */
    uint32_t *offsets;    /* query offsets */
    uint32_t n_offsets;
} orc_lookup;

extern const int32_t ORC_BLOSUM62[ORC_ALPHABET][ORC_ALPHABET];

int orc_lookup_build(const uint8_t *query, int32_t qlen, int32_t threshold, orc_lookup *out);
void orc_lookup_free(orc_lookup *lk);

/* Word finder + ungapped stage for one subject. Writes up to cap init hits in
 * the order the gapped stage visits them; returns the total count. */
int32_t orc_subject_inits(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                          const uint8_t *subj, int32_t slen, uint32_t subject_index,
                          const orc_params *p, orc_init *out, int32_t cap);

/* Full preliminary stage for one subject (before E-values). Writes up to cap
 * HSPs in final per-subject order; returns the total count. */
int32_t orc_subject_hsps(const uint8_t *query, int32_t qlen, const orc_lookup *lk,
                         const uint8_t *subj, int32_t slen, uint32_t subject_index,
                         const orc_params *p, orc_hsp *out, int32_t cap);

/* Score-only semi-gapped X-drop alignment (exposed for unit tests).
 * reverse=0: rows A[1..M], columns B[1..N]; reverse=1: rows A[M-1..0],
 * columns B[N-1..0]. */
int32_t orc_semi_gapped(const uint8_t *A, const uint8_t *B, int32_t M, int32_t N, int32_t reverse,
                        int32_t gap_open, int32_t gap_extend, int32_t xdrop,
                        int32_t *a_best, int32_t *b_best);

/* Gapped start point over the 11-residue window (exposed for unit tests). */
int32_t orc_gapped_start(const uint8_t *q, const uint8_t *s, int32_t q_start, int32_t s_start,
                         int32_t len);

/* Whole database, multithreaded over subjects. Subjects are
 * residues[offsets[i] .. offsets[i+1]). Results are ordered by subject index.
 * Returns an opaque handle (NULL on allocation failure). */
typedef struct orc_result orc_result;
orc_result *orc_search_db(const uint8_t *query, int32_t qlen, const uint8_t *residues,
                          const uint64_t *offsets, uint32_t n_subjects, const orc_params *p,
                          int32_t n_threads, int32_t want_inits);
uint64_t orc_result_n_hsps(const orc_result *r);
uint64_t orc_result_n_inits(const orc_result *r);
void orc_result_copy_hsps(const orc_result *r, orc_hsp *out);
void orc_result_copy_inits(const orc_result *r, orc_init *out);
void orc_result_free(orc_result *r);

/* Traceback of one gapped HSP (the published gapped-BLAST traceback:
 * X-drop alignment left and right of the start point with the path kept).
 * The DP is the banded X-drop DP above with the final X-drop; each live cell
 * records where its score came from (diagonal beats a vertical gap beats a
 * horizontal gap on ties; a gap state extends rather than opens on ties);
 * the path runs back from the first best cell to the origin. */
typedef struct orc_tb {
    int32_t score;
    int32_t q_start, q_end, s_start, s_end;  /* 0-based, ends exclusive */
    int32_t length;                          /* aligned columns */
    int32_t identities, positives, mismatches;
    int32_t gap_opens, gaps;
} orc_tb;
int orc_traceback(const uint8_t *query, int32_t qlen, const uint8_t *subject, int32_t slen, int32_t q_off,
                  int32_t s_off, int32_t gap_open, int32_t gap_extend, int32_t xdrop, orc_tb *out);
/* The same, also writing the alignment's moves in query order ('M' pair,
 * 'I' query residue against a gap, 'D' subject residue against a gap). */
int orc_traceback_ops(const uint8_t *query, int32_t qlen, const uint8_t *subject, int32_t slen, int32_t q_off,
                      int32_t s_off, int32_t gap_open, int32_t gap_extend, int32_t xdrop, orc_tb *out, char *ops,
                      int32_t ops_cap, int32_t *n_ops);

/* Karlin-Altschul arithmetic (restated published formulas). */
double orc_evalue(int32_t score, double lambda, double K, double searchsp);
int32_t orc_length_adjustment(double K, double logK, double alpha_d_lambda, double beta,
                              int32_t query_length, int64_t db_length, int64_t db_num_seqs);

#ifdef __cplusplus
}
#endif
#endif
