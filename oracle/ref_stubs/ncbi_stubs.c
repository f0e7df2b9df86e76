/* Bodies for the stub BlastSeqSrc declarations (ref_stubs/algo/blast/core/
 * blast_seqsrc.h), so that the reference's BLAZE_gpu sources link into the
 * oracle's cross-check library. None of them is called: the cross-check
 * calls the reference's lookup construction and kernels directly. Each one
 * reports failure or leaves its outputs empty. Test infrastructure only. */
#include <stddef.h>

#include "algo/blast/core/blast_seqsrc.h"

int32_t BlastSeqSrcGetNumSeqs(const BlastSeqSrc *s) { (void)s; return 0; }
int16_t BlastSeqSrcGetSequence(const BlastSeqSrc *s, BlastSeqSrcGetSeqArg *a) { (void)s; (void)a; return -1; }
void BlastSeqSrcReleaseSequence(const BlastSeqSrc *s, BlastSeqSrcGetSeqArg *a) { (void)s; (void)a; }
void BlastSeqSrcGetDBPointer(BlastSeqSrc *s, char **p) { (void)s; *p = NULL; }
void BlastSeqSrcGetQueryPointers(BlastSeqSrc *s, char **a, char **b) { (void)s; *a = *b = NULL; }
void BlastSeqSrcGetDBWorkInfoGPU(BlastSeqSrc *s, uint64_t **a, uint64_t *b, uint64_t *c, uint64_t **d, uint64_t **e,
                                 uint64_t **f) {
    (void)s;
    *a = *d = *e = *f = NULL;
    *b = *c = 0;
}
void BlastSeqSrcGetIsolationPointers(BlastSeqSrc *s, uint16_t **a, uint16_t **b, uint16_t **c) {
    (void)s;
    *a = *b = *c = NULL;
}
void BlastSeqSrcGetHostDBPointer(BlastSeqSrc *s, char **p) { (void)s; *p = NULL; }
void BlastSeqSrcGetSequenceBitmaskPointer(BlastSeqSrc *s, char **p) { (void)s; *p = NULL; }
