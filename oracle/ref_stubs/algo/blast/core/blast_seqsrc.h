/* Stub for building the reference's BLAZE_gpu sources as the oracle's
 * cross-check (test infrastructure only). It declares just enough of NCBI's
 * BlastSeqSrc interface, and of the BLAZE accessors added to it, for the
 * reference's host driver BLAZE_GPU (BLAZE_gpu/gpuBLAZE.cu:1428-1704) to
 * compile; the cross-check never calls that driver, and ncbi_stubs.c gives
 * the accessors bodies that only report failure. Shapes follow their call
 * sites in gpuBLAZE.cu and BLAZE_ncbi/blast_seqsrc.h:336-451. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct BlastSeqSrc BlastSeqSrc;

typedef struct BLAST_SequenceBlk {
    uint8_t *sequence;
    int32_t length;
} BLAST_SequenceBlk;

typedef enum { eBlastEncodingProtein = 0 } EBlastEncoding;

typedef struct BlastSeqSrcGetSeqArg {
    int32_t oid;
    EBlastEncoding encoding;
    int check_oid_exclusion;
    BLAST_SequenceBlk *seq;
} BlastSeqSrcGetSeqArg;

int32_t BlastSeqSrcGetNumSeqs(const BlastSeqSrc *seq_src);
int16_t BlastSeqSrcGetSequence(const BlastSeqSrc *seq_src, BlastSeqSrcGetSeqArg *arg);
void BlastSeqSrcReleaseSequence(const BlastSeqSrc *seq_src, BlastSeqSrcGetSeqArg *arg);
void BlastSeqSrcGetDBPointer(BlastSeqSrc *seq_src, char **db);
void BlastSeqSrcGetQueryPointers(BlastSeqSrc *seq_src, char **query_db, char **query);
void BlastSeqSrcGetDBWorkInfoGPU(BlastSeqSrc *seq_src, uint64_t **prefix_index, uint64_t *index_size,
                                 uint64_t *num_chunks, uint64_t **chunk_start, uint64_t **chunk_end,
                                 uint64_t **db_offset);
void BlastSeqSrcGetIsolationPointers(BlastSeqSrc *seq_src, uint16_t **lookup, uint16_t **offsets,
                                     uint16_t **seeds);
void BlastSeqSrcGetHostDBPointer(BlastSeqSrc *seq_src, char **host_db);
void BlastSeqSrcGetSequenceBitmaskPointer(BlastSeqSrc *seq_src, char **bitmask);

#ifdef __cplusplus
}
#endif
