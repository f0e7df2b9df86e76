/*
 * blaze_prelim.h -- C ABI of libblaze103, a GB300 (sm_103a) implementation of
 * the BLASTP preliminary search stage (word lookup -> two-hit seeds ->
 * ungapped X-drop -> semi-gapped X-drop -> per-subject HSP lists).
 *
 * Plain pointers and sizes only. Every entry point returns a blaze_status
 * (0 = success), never exits the process and lets no C++ exception out (a
 * failed host allocation is BLAZE_ERR_OUT_OF_MEMORY). Handles are not thread-safe;
 * use one blaze_search per host thread (each owns its CUDA stream).
 *
 * Reference interfaces replaced (paths within 181charan/BLAZE-SC-ad):
 *   BLAZE_GPU(seq_src, threadIndex, totalThreads, queryLen, survivingSeqs,
 *             num_survivors, ungapped_cutoff, gapped_cutoff)
 *       BLAZE_gpu/gpu_cpu_common.h:43, BLAZE_gpu/gpuBLAZE.cu:1428-1704
 *     -> blaze_search_run + blaze_search_results: instead of a survivor
 *        list that the CPU re-searches (blast_engine.c:2223-2558), the GPU
 *        returns each subject's finished HSP list.
 *   copyConstantMemory / deviceAlloc / deviceMemCpyToDevice of the query
 *   tables (gpu_cpu_common.h:63-70, prelim_stage.cpp:340-571)
 *     -> blaze_query_create.
 *   The per-thread DB gathers through BlastSeqSrcGetSequence and the staging
 *   buffers (prelim_stage.cpp:478-1229, gpuBLAZE.cu:1587-1618)
 *     -> blaze_db_create: one length-sorted, device-resident copy.
 *   BlastInitialWordParametersNew / BlastHitSavingParameters cutoffs
 *   (blast_engine.c:2971-2981) -> blaze_params_default (the caller may pass
 *   NCBI's own values instead).
 */
#ifndef BLAZE_PRELIM_H
#define BLAZE_PRELIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum blaze_status {
    BLAZE_OK = 0,
    BLAZE_ERR_INVALID_ARG = 1,   /* bad pointer, size or residue code */
    BLAZE_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    BLAZE_ERR_NO_DEVICE = 3,     /* no usable GPU */
    BLAZE_ERR_OUT_OF_MEMORY = 4, /* device or host allocation failed */
    BLAZE_ERR_OUTPUT_TOO_SMALL = 5, /* caller buffer too small; count reported */
    BLAZE_ERR_LIMIT = 6,         /* request exceeds a documented limit */
    BLAZE_ERR_INTERNAL = 7       /* a device-side consistency check failed */
} blaze_status;

typedef struct blaze_db blaze_db;         /* resident residue database */
typedef struct blaze_query blaze_query;   /* query + word lookup on the device */
typedef struct blaze_search blaze_search; /* stream, scratch and results */
typedef struct blaze_batch blaze_batch;   /* many queries' tables on the device */

/* Search parameters. Raw scores; NCBI BLAST defaults for BLOSUM62 11/1 are
 * word_threshold 11, window 40, ungapped_xdrop 16, gap_open 11,
 * gap_extend 1, gapped_xdrop 38. */
typedef struct blaze_params {
    int32_t word_threshold;
    int32_t window;
    int32_t ungapped_xdrop;
    int32_t ungapped_cutoff; /* word_params->cutoffs->cutoff_score */
    int32_t gap_open;
    int32_t gap_extend;
    int32_t gapped_xdrop;
    int32_t gapped_cutoff;   /* hit_params->cutoffs->cutoff_score */
    double lambda;           /* gapped Karlin-Altschul lambda */
    double K;                /* gapped Karlin-Altschul K */
    double eff_searchsp;     /* effective search space of the query */
    double prelim_evalue;    /* HSPs with a larger E-value are dropped */
    /* Culling of the returned lists, on the device (0: none). hitlist_size
     * (NCBI max_target_seqs): per query, the subjects with the best E-values,
     * ties by smaller OID. max_hsps: per subject, the first HSPs of its list.
     * lambda, K and eff_searchsp must be finite with lambda, K > 0 and
     * eff_searchsp >= 0 (BLAZE_ERR_INVALID_ARG otherwise). */
    int32_t hitlist_size;
    int32_t max_hsps;
} blaze_params;

/* One HSP of a subject; offsets 0-based, ends exclusive (NCBI BlastHSP's
 * query.offset/end, subject.offset/end, score, evalue, and the gapped start
 * point). */
typedef struct blaze_hsp {
    uint32_t oid;
    int32_t score;
    int32_t q_start, q_end;
    int32_t s_start, s_end;
    int32_t q_gapped_start, s_gapped_start;
    double evalue;
} blaze_hsp;

/* An ungapped HSP that reached the ungapped cutoff and went on to the gapped
 * stage (NCBI BlastInitHSP: ungapped_data plus the triggering word hit). */
typedef struct blaze_init_hit {
    uint32_t oid;
    int32_t q_start, s_start, length, score;
    int32_t q_trigger, s_trigger;
} blaze_init_hit;

/* Counters of the last run (diagnostics; NCBI BlastDiagnostics analog). */
typedef struct blaze_stats {
    uint64_t residues_scanned;
    uint64_t word_hits;
    uint64_t ungapped_extensions;
    uint64_t init_hsps;
    uint64_t gapped_extensions;
    uint64_t dp_cells;
    uint64_t hsps;
    uint32_t subjects_with_hsps;
    uint32_t reruns; /* device buffers grown and the pass repeated */
    /* CUDA-event times on the search stream, last pass only (milliseconds) */
    float scan_ms;   /* word finder + ungapped kernel */
    float gapped_ms; /* gapped kernel */
    float device_ms; /* first to last device operation of the run, all passes */
    uint32_t kernel_launches; /* kernels launched by the run, all passes */
    uint64_t h2d_bytes; /* host->device bytes of the run (query tables included) */
    uint64_t d2h_bytes; /* device->host bytes of the run */
    uint32_t graph_replays; /* passes launched from an already built CUDA graph */
    uint32_t graph_builds;  /* passes that captured (or updated) the CUDA graph */
    float traceback_ms;     /* last blaze_search_traceback: its kernel launches (CUDA events) */
    uint32_t traceback_hsps;
    uint64_t traceback_cells; /* DP cells of the traceback (left and right, all passes) */
} blaze_stats;

const char *blaze_status_string(int status);

/* Text of the last CUDA runtime error seen by this thread inside the library
 * ("no error" when none); explains a BLAZE_ERR_CUDA status. */
const char *blaze_last_cuda_error(void);

/* Number of usable devices (0 when none). */
int blaze_device_count(int *count);

/* Database: residues[offsets[i] .. offsets[i+1]) is subject i (its OID).
 * NCBIstdaa codes 1..27; subjects of any length >= 0. The library keeps a
 * length-sorted copy in device memory. */
int blaze_db_create(int device, const uint8_t *residues, const uint64_t *offsets,
                    uint32_t n_subjects, blaze_db **out);
int blaze_db_free(blaze_db *db);
int blaze_db_info(const blaze_db *db, uint64_t *total_residues, uint32_t *n_subjects,
                  uint32_t *max_length);

/* A database source shaped like NCBI's BlastSeqSrc, so that an engine that
 * already holds a BlastSeqSrc* hands it over through a thin adapter
 * (function pointers plus a user pointer; BLAZE_ncbi/blast_seqsrc.c:91-130 and
 * the accessors BlastSeqSrcGetNumSeqs, GetTotLen, GetMaxSeqLen, GetSeqLen,
 * GetSequence :325-333, ReleaseSequence, IteratorNext). It replaces the
 * reference GPU driver's per-chunk gathers through BlastSeqSrcGetSequence
 * (BLAZE_gpu/gpuBLAZE.cu:1587-1611): the library reads every sequence once,
 * on the calling thread, into its resident length-sorted copy.
 *
 *   get_num_seqs      number of OIDs (>= 0); required
 *   get_sequence      residues of `oid` (NCBIstdaa codes 1..27, no sentinel
 *                     bytes) and their count; the pointer stays valid until
 *                     release_sequence(oid) or the next get_sequence; returns
 *                     0 on success; required
 *   release_sequence  called after each get_sequence (may be NULL)
 *   get_seq_len       length of `oid` without fetching it (may be NULL: the
 *                     lengths are then taken from a first get_sequence pass)
 *   get_tot_len, get_max_seq_len
 *                     may be NULL; when given (and iter_next is NULL), they
 *                     must equal the total and the largest length read
 *   iter_next         the next OID to search, negative at the end (NCBI's
 *                     BLAST_SEQSRC_EOF); may be NULL: every OID. OIDs the
 *                     iterator does not return stay in the database as empty
 *                     subjects, so OID numbering is kept.
 * A callback error, a length that disagrees between calls, an OID out of
 * range or returned twice by iter_next, a residue code outside 1..27 or
 * totals that disagree return BLAZE_ERR_INVALID_ARG and create nothing. */
typedef struct blaze_seq_source {
    void *user;
    int64_t (*get_num_seqs)(void *user);
    int (*get_sequence)(void *user, uint32_t oid, const uint8_t **residues, uint32_t *length);
    void (*release_sequence)(void *user, uint32_t oid);
    int64_t (*get_seq_len)(void *user, uint32_t oid);
    int64_t (*get_tot_len)(void *user);
    int64_t (*get_max_seq_len)(void *user);
    int64_t (*iter_next)(void *user);
} blaze_seq_source;
int blaze_db_create_from_source(int device, const blaze_seq_source *src, blaze_db **out);

/* NCBI BLAST protein database volume: `path` without extension names the
 * <path>.pin index and <path>.psq sequence file (format versions 4 and 5).
 * OID i of the volume becomes subject i. Replaces the per-subject
 * BlastSeqSrcGetSequence gathers of the reference's GPU driver
 * (BLAZE_gpu/gpuBLAZE.cu:1587-1611). Malformed or non-protein volumes return
 * BLAZE_ERR_INVALID_ARG. */
int blaze_volume_info(const char *path, uint32_t *n_subjects, uint64_t *total_residues,
                      uint32_t *max_length);
/* Residues of every sequence, concatenated without separators, and n+1
 * offsets (capacity: residues bytes available). */
int blaze_volume_read(const char *path, uint8_t *residues, uint64_t capacity, uint64_t *offsets);
/* blaze_volume_read + blaze_db_create. */
int blaze_db_open(int device, const char *path, blaze_db **out);

/* Query: NCBIstdaa codes 1..27, 1 <= length <= 32000. Builds the word lookup
 * (every word scoring >= word_threshold against a query word, plus the query
 * word itself) and uploads it. */
int blaze_query_create(const blaze_db *db, const uint8_t *query, int32_t length,
                       int32_t word_threshold, blaze_query **out);
int blaze_query_free(blaze_query *q);

/* NCBI BLAST defaults for a blastp search of one query against db with the
 * given expect value: cutoffs, X-drops, effective search space (length
 * adjustment of Altschul & Gish), Karlin-Altschul constants. */
int blaze_params_default(int32_t query_length, uint64_t db_residues, uint32_t db_subjects,
                         double evalue, blaze_params *out);

int blaze_search_create(blaze_db *db, blaze_search **out);
int blaze_search_free(blaze_search *s);

/* Runs the preliminary stage of query q against the whole database on the
 * GPU. On return the results are held by s; *n_hsps is their count. */
int blaze_search_run(blaze_search *s, const blaze_query *q, const blaze_params *p,
                     uint64_t *n_hsps);

/* Copies the results of the last run, grouped by OID (ascending) and, within
 * an OID, in NCBI's per-subject order (score descending). Returns
 * BLAZE_ERR_OUTPUT_TOO_SMALL when capacity < count (nothing copied). */
int blaze_search_results(const blaze_search *s, blaze_hsp *out, uint64_t capacity,
                         uint64_t *n_hsps);
int blaze_search_stats(const blaze_search *s, blaze_stats *out);

/* Diagnostics: the init hits of the last single-query run, grouped by OID (ascending) and
 * in the order the gapped stage visits them (score descending, then subject
 * and query offset of the trigger). Same capacity rule as above. */
int blaze_search_init_hits(blaze_search *s, blaze_init_hit *out, uint64_t capacity,
                           uint64_t *n_hits);

/* ---------------------------------------------------------------------
 * Traceback stage (after the preliminary search; NCBI's traceback of
 * BLAZE_ncbi/prelim_stage.cpp:1462-1498): every HSP of the last single-query
 * run of s is aligned again from its gapped start point with the final
 * X-drop (NCBI blastp: 64 = 25 bits), keeping the path; per subject,
 * duplicates are purged and the list sorted as in the preliminary stage;
 * E-values come from the final scores and HSPs above `evalue` are dropped.
 * q must hold the query of that run. */
typedef struct blaze_aligned_hsp {
    uint32_t oid;
    int32_t score;
    int32_t q_start, q_end, s_start, s_end; /* 0-based, ends exclusive */
    int32_t length;                         /* aligned columns */
    int32_t identities, positives, mismatches, gap_opens, gaps;
    int32_t reserved;
    double evalue;
    double bit_score;                       /* (lambda * score - ln K) / ln 2 */
} blaze_aligned_hsp;
int blaze_search_traceback(blaze_search *s, const blaze_query *q, const blaze_params *params, int32_t final_xdrop,
                           double evalue, uint64_t *n_hsps);
/* Results of the last traceback, by OID, then the final per-subject order. */
int blaze_search_traceback_results(const blaze_search *s, blaze_aligned_hsp *out, uint64_t capacity,
                                   uint64_t *n_hsps);

/* The same for the last batched run of s, which must have searched b with
 * `params` (one set per query): records by query, then OID. */
typedef struct blaze_batch_aligned_hsp {
    uint32_t query;
    uint32_t reserved;
    blaze_aligned_hsp hsp;
} blaze_batch_aligned_hsp;
int blaze_search_traceback_batch(blaze_search *s, const blaze_batch *b, const blaze_params *params,
                                 int32_t final_xdrop, double evalue, uint64_t *n_hsps);
int blaze_search_traceback_batch_results(const blaze_search *s, blaze_batch_aligned_hsp *out, uint64_t capacity,
                                         uint64_t *n_hsps);

/* ---------------------------------------------------------------------
 * Batched form: many queries of uneven length against the database in one
 * persistent launch per stage. Warps pull (query, subject range) tiles from a
 * device work queue, longest subjects first, queries interleaved. All
 * queries of a batch share word_threshold, window, X-drops and gap costs;
 * cutoffs and E-value statistics are per query (params[i]).
 */

/* One HSP of a batched run: the query's index in the batch and the HSP. */
typedef struct blaze_batch_hsp {
    uint32_t query;
    uint32_t reserved;
    blaze_hsp hsp;
} blaze_batch_hsp;

/* Queries residues[offsets[i] .. offsets[i+1]), i < n_queries, each valid as
 * for blaze_query_create. */
int blaze_batch_create(const blaze_db *db, const uint8_t *residues, const uint64_t *offsets,
                       uint32_t n_queries, int32_t word_threshold, blaze_batch **out);
int blaze_batch_free(blaze_batch *b);
/* Device memory the batch's tables take (the serving loop admits by it). */
int blaze_batch_info(const blaze_batch *b, uint32_t *n_queries, uint64_t *device_bytes);

/* Runs every query of b; params points to n_queries parameter sets. Results
 * are held by s until the next run. */
int blaze_search_run_batch(blaze_search *s, const blaze_batch *b, const blaze_params *params,
                           uint64_t *n_hsps);
/* Results of the last batched run, grouped by query, then OID (ascending),
 * then NCBI's per-subject order. Same capacity rule as blaze_search_results. */
int blaze_search_batch_results(const blaze_search *s, blaze_batch_hsp *out, uint64_t capacity,
                               uint64_t *n_hsps);

/* Launch shape of the word finder (0 = library default): subjects up to
 * stage_bytes residues are staged in shared memory; a batched tile is one
 * block's work for one query: consecutive subjects of about tile_residues
 * residues per warp of the block (a longer subject is a tile of its own; 0:
 * sized so that every warp gets several tiles' worth); max_warps_per_block
 * caps the block. */
typedef struct blaze_tuning {
    uint32_t stage_bytes;
    uint32_t tile_residues;
    uint32_t max_warps_per_block;
    /* 0: the per-pass launch sequence (counter reset, scan, gapped, counter
     * read-back) runs as a CUDA graph for batched runs and as direct launches
     * for single queries; 1: direct launches always; 2: CUDA graph always.
     * The graph is captured once and replayed while the launch arguments stay
     * the same (updated in place when they change). */
    uint32_t launch_mode;
    /* Batched runs: 0: automatic (one scan launch per query for batches of
     * at most 16 queries or databases from 2^27 residues on, where a query
     * alone fills the GPU; tiles of many queries per launch otherwise);
     * 1: tiles always; 2: one launch per query always. Results are
     * identical either way. */
    uint32_t batch_launch;
} blaze_tuning;
int blaze_search_set_tuning(blaze_search *s, const blaze_tuning *t);

/* ---------------------------------------------------------------------
 * Serving loop: continuous batching over the resident database. Queries are
 * submitted as they arrive; `slots` worker threads (each with its own search
 * context and CUDA stream) take the waiting queries into their next batch
 * as soon as they are free, admitting queries while the device memory of
 * the in-flight batches (word tables plus a per-query allowance for seed and
 * HSP buffers) stays within memory_budget, so batches overlap on the GPU.
 * Each query's HSP lists are handed back when its batch completes. On a
 * database of 2^27 residues or more (unless tuning.batch_launch forces
 * tiles), where a batched run launches the word finder once per query and a
 * query alone fills the GPU, batches take at most 4 queries and run on the
 * GPU one at a time (the workers' host work still overlaps): batching saves
 * nothing there, and concurrent whole-GPU launches only contend.
 */
typedef struct blaze_server blaze_server;

typedef struct blaze_server_config {
    uint32_t slots;           /* batches in flight at once (1..64; BLAZE_ERR_LIMIT above) */
    uint32_t max_batch;       /* queries per batch at most (>= 1) */
    uint64_t memory_budget;   /* bytes for in-flight batches (0: no limit) */
    uint32_t batch_window_us; /* after the first waiting query, wait this long for more */
    double evalue;            /* expect value for every query's default parameters */
    blaze_tuning tuning;      /* launch shape of every worker's search (zeros: defaults) */
} blaze_server_config;

typedef struct blaze_server_stats {
    uint64_t submitted, completed, batches;
    uint64_t residues;        /* query x database residues completed */
    double latency_p50_ms, latency_p99_ms, latency_max_ms;
    double busy_s;            /* wall time from first submit to last completion */
} blaze_server_stats;

int blaze_server_create(blaze_db *db, const blaze_server_config *cfg, blaze_server **out);
/* Queues one query; *ticket identifies it. Thread-safe. */
int blaze_server_submit(blaze_server *srv, const uint8_t *query, int32_t length, uint64_t *ticket);
/* Blocks until the ticket's batch completed (timeout_ms < 0: no limit);
 * returns BLAZE_ERR_LIMIT on timeout. *n_hsps is its HSP count. */
int blaze_server_wait(blaze_server *srv, uint64_t ticket, int32_t timeout_ms, uint64_t *n_hsps);
/* Copies a completed ticket's HSPs (grouped by OID, NCBI order), its latency
 * from submission to completion, and releases the ticket. */
int blaze_server_take(blaze_server *srv, uint64_t ticket, blaze_hsp *out, uint64_t capacity,
                      uint64_t *n_hsps, double *latency_ms);
int blaze_server_stats_get(blaze_server *srv, blaze_server_stats *out);
/* Finishes every queued query, stops the workers and frees the server. */
int blaze_server_free(blaze_server *srv);

/* Convenience: blaze_query_create + blaze_search_run + blaze_search_results
 * in one call with host buffers (the drop-in path). */
int blaze_prelim_search(blaze_search *s, const uint8_t *query, int32_t length,
                        const blaze_params *p, blaze_hsp *out, uint64_t capacity,
                        uint64_t *n_hsps);

/* ---------------------------------------------------------------------
 * Gapped stage without device allocation.
 *
 * This entry point has no counterpart in the reference. It serves callers
 * that cannot call cudaMalloc: applications whose own allocator already owns
 * the device heap, and code that must not allocate because cudaMalloc and
 * cudaFree can synchronize the whole device and stall other streams. The
 * caller passes all inputs and outputs in its own device memory; the working
 * memory (DP rows, ordered init hits, kept HSPs, counters) is one fixed
 * array of BLAZE_NOALLOC_SCRATCH_BYTES compiled into the library, which every
 * GPU that loads the library holds until the process exits.
 *
 * Input: the ungapped HSPs of each subject (d_init_hits, any order within a
 * subject), grouped by d_subjects[i] = {subject index into d_offsets, count,
 * first record}. Output: finished HSPs (score order within a subject,
 * subjects in any order) in d_out; d_result[0] = HSPs produced (more than
 * out_capacity means the output was cut), d_result[1] = status bits
 * (0 = complete; BLAZE_NOALLOC_* below). Every subject must be at most
 * max_subject_length residues long and carry at most
 * max_init_hits_per_subject init hits; values above
 * BLAZE_NOALLOC_MAX_SUBJECT_LENGTH / BLAZE_NOALLOC_MAX_INIT_HITS are rejected
 * with BLAZE_ERR_LIMIT. The device checks each subject and init hit again:
 * a subject longer than BLAZE_NOALLOC_MAX_SUBJECT_LENGTH or with more than
 * BLAZE_NOALLOC_MAX_INIT_HITS init hits is skipped, and so is an init hit
 * that does not lie inside the query and its subject (length >= 1); each
 * such skip sets its status bit and the other subjects' HSPs are unchanged.
 * Subject indices are not checked (the library does not know how many
 * offsets d_offsets holds): each must be below that count.
 *
 * The call only enqueues work on `stream` (a cudaStream_t); read d_result
 * after synchronizing it. The first call on a device looks up the device
 * address of the fixed array, so make that first call before any stream
 * capture; the address is kept per CUDA context, so after a device reset
 * (cudaDeviceReset) the next call looks it up again and should likewise come
 * before any capture. All calls share the one array: calls whose work overlaps on the
 * GPU (other streams, other threads) race and must be serialized by the
 * caller. */
#define BLAZE_NOALLOC_MAX_SUBJECT_LENGTH 4096u
#define BLAZE_NOALLOC_MAX_INIT_HITS 128u
#define BLAZE_NOALLOC_SCRATCH_BYTES (12u << 20)
/* status bits of d_result[1] */
#define BLAZE_NOALLOC_OUTPUT_CUT 4u          /* more HSPs than out_capacity */
#define BLAZE_NOALLOC_TOO_MANY_INIT_HITS 16u /* a subject with too many init hits was skipped */
#define BLAZE_NOALLOC_SUBJECT_TOO_LONG 32u   /* a subject over the length maximum was skipped */
#define BLAZE_NOALLOC_BAD_INIT_HIT 64u       /* an init hit outside its sequences was skipped */

typedef struct blaze_dev_init_hit {
    int32_t q_start, s_start, length, score;
    int32_t q_trigger, s_trigger;
} blaze_dev_init_hit;

typedef struct blaze_dev_subject {
    uint32_t subject;
    uint32_t n_init_hits;
    uint64_t first_init_hit;
} blaze_dev_subject;

typedef struct blaze_dev_hsp {
    uint32_t subject;
    int32_t score, q_start, q_end, s_start, s_end, q_gapped_start, s_gapped_start;
} blaze_dev_hsp;

int blaze_gapped_noalloc(const uint8_t *d_residues, const uint64_t *d_offsets,
                         uint32_t max_subject_length, const uint8_t *d_query,
                         int32_t query_length, const blaze_dev_init_hit *d_init_hits,
                         const blaze_dev_subject *d_subjects, uint32_t n_subjects,
                         uint32_t max_init_hits_per_subject, const blaze_params *p,
                         blaze_dev_hsp *d_out, uint64_t out_capacity, uint64_t *d_result,
                         void *stream);

#ifdef __cplusplus
}
#endif
#endif
