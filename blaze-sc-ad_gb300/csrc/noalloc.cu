// noalloc.cu -- the gapped stage without any device allocation.
//
// For callers that cannot call cudaMalloc: hosts whose own allocator owns the
// whole device heap, and code paths where an allocation is not allowed
// because cudaMalloc/cudaFree may synchronize the device and stall work on
// other streams. The caller passes every input and output in its own device
// memory; the kernel's working memory is one fixed array compiled into this
// library (BLAZE_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the
// library until the process exits).
#include <cstddef>
#include <mutex>

#include "common.cuh"

using namespace blaze;

namespace {

// Fixed shape of the gapped kernel in this mode: 304 warps, as 152 blocks of
// two warps so that every SM of a GB300 takes a share of the work.
constexpr int kWarpsPerBlock = 2;
constexpr int kBlocks = 152;
constexpr int kWarps = kBlocks * kWarpsPerBlock;                         // 304
constexpr uint32_t kMaxInit = BLAZE_NOALLOC_MAX_INIT_HITS;             // per subject
constexpr uint32_t kDpStride = BLAZE_NOALLOC_MAX_SUBJECT_LENGTH + 2;   // ints per DP row
constexpr size_t kCountersBytes = 256;
constexpr size_t kSortedBytes = sizeof(InitHit) * kWarps * kMaxInit;
constexpr size_t kSavedBytes = sizeof(DevHsp) * kWarps * kMaxInit;
constexpr size_t kDpBytes = sizeof(int32_t) * 2ull * kWarps * kDpStride;
constexpr size_t kScratchBytes = kCountersBytes + kSortedBytes + kSavedBytes + kDpBytes;
static_assert(kScratchBytes <= BLAZE_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");
static_assert(sizeof(DevCounters) <= kCountersBytes, "counters");
static_assert(sizeof(blaze_dev_init_hit) == sizeof(InitHit), "init hit layout");
static_assert(sizeof(blaze_dev_subject) == sizeof(WorkItem), "subject group layout");
static_assert(sizeof(blaze_dev_hsp) == sizeof(DevHsp), "HSP layout");
static_assert(offsetof(blaze_dev_subject, first_init_hit) == offsetof(WorkItem, first), "group layout");
static_assert(BLAZE_NOALLOC_OUTPUT_CUT == kFlagOutArrayFull && BLAZE_NOALLOC_TOO_MANY_INIT_HITS == kFlagBadState &&
                  BLAZE_NOALLOC_SUBJECT_TOO_LONG == kFlagSubjectTooLong &&
                  BLAZE_NOALLOC_BAD_INIT_HIT == kFlagBadInitHit,
              "status bits of d_result[1]");

// The working memory of every call, on every device that loads the library.
static __device__ __align__(256) unsigned char g_noalloc_scratch[BLAZE_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch, looked up once per CUDA context: the
// cache is keyed by the context's process-unique ID, so a context that was
// destroyed (cudaDeviceReset) and created again gets a fresh lookup. The
// driver's context calls are reached through the runtime's entry-point
// query, so the library links no driver library.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

using CtxGetCurrentFn = int (*)(void **ctx);
using CtxGetIdFn = int (*)(void *ctx, unsigned long long *id);

int current_context_id(unsigned long long *id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult r1{}, r2{};
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &r1);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &r2);
        if (e != cudaSuccess) {
            last_cuda_error(e);
            return BLAZE_ERR_CUDA;
        }
        if (r1 != cudaDriverEntryPointSuccess || r2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return BLAZE_ERR_CUDA;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void *ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, id) != 0) return BLAZE_ERR_CUDA;
    return BLAZE_OK;
}

// Called with `device` current. A cached address is reused only while the
// current context is the one it was looked up in; the first lookup of a
// context goes through cudaGetSymbolAddress, which also initialises the
// context when nothing has yet.
int scratch_address(int device, unsigned char **out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long ctx = 0;
    if (g_scratch_addr[device]) {
        int rc = current_context_id(&ctx);
        if (rc != BLAZE_OK) return rc;
        if (ctx == g_scratch_ctx[device]) {
            *out = g_scratch_addr[device];
            return BLAZE_OK;
        }
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // creates the context if needed
    if (e != cudaSuccess) {
        last_cuda_error(e);
        return BLAZE_ERR_CUDA;
    }
    int rc = current_context_id(&ctx);
    if (rc != BLAZE_OK) return rc;
    g_scratch_addr[device] = static_cast<unsigned char *>(p);
    g_scratch_ctx[device] = ctx;
    *out = g_scratch_addr[device];
    return BLAZE_OK;
}

}  // namespace

extern "C" int blaze_gapped_noalloc(const uint8_t *d_residues, const uint64_t *d_offsets,
                                    uint32_t max_subject_length, const uint8_t *d_query,
                                    int32_t query_length, const blaze_dev_init_hit *d_init_hits,
                                    const blaze_dev_subject *d_subjects, uint32_t n_subjects,
                                    uint32_t max_init_hits_per_subject, const blaze_params *p,
                                    blaze_dev_hsp *d_out, uint64_t out_capacity,
                                    uint64_t *d_result, void *stream) {
    if (!d_residues || !d_offsets || !d_query || query_length <= 0 || !p || !d_result ||
        (n_subjects > 0 && (!d_init_hits || !d_subjects)) || (out_capacity > 0 && !d_out))
        return BLAZE_ERR_INVALID_ARG;
    if (p->gap_open < 0 || p->gap_extend <= 0 || p->gapped_xdrop <= 0 || p->gapped_cutoff <= 0)
        return BLAZE_ERR_INVALID_ARG;
    if (max_subject_length > BLAZE_NOALLOC_MAX_SUBJECT_LENGTH ||
        max_init_hits_per_subject > BLAZE_NOALLOC_MAX_INIT_HITS)
        return BLAZE_ERR_LIMIT;
    int device = 0;
    BLAZE_CUDA_TRY(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) return BLAZE_ERR_LIMIT;
    unsigned char *base = nullptr;
    int rc = scratch_address(device, &base);
    if (rc != BLAZE_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto *cnt = reinterpret_cast<DevCounters *>(base);

    // everything the kernel counts must start at zero; the work count is set
    // to all ones so that the kernel takes n_subjects (its cap) as the count
    BLAZE_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(DevCounters), st));
    BLAZE_CUDA_TRY(cudaMemsetAsync(&cnt->work_count, 0xff, sizeof(cnt->work_count), st));
    BLAZE_CUDA_TRY(cudaMemsetAsync(d_result, 0, 2 * sizeof(uint64_t), st));

    GappedArgs ga{};
    ga.res = d_residues;
    ga.off = d_offsets;
    ga.q = d_query;
    ga.qlen = query_length;
    ga.init_in = reinterpret_cast<const InitHit *>(d_init_hits);
    ga.work = reinterpret_cast<const WorkItem *>(d_subjects);
    ga.work_cap = n_subjects;
    ga.init_cap = ~0ull;  // the caller's arrays: sizes unknown here
    ga.n_subj = ~0u;
    ga.n_queries = 1;
    ga.sorted = reinterpret_cast<InitHit *>(base + kCountersBytes);
    ga.saved = reinterpret_cast<DevHsp *>(base + kCountersBytes + kSortedBytes);
    ga.cap = kMaxInit;
    ga.dp = reinterpret_cast<int32_t *>(base + kCountersBytes + kSortedBytes + kSavedBytes);
    ga.dp_stride = kDpStride;
    ga.gap_open = p->gap_open;
    ga.gap_extend = p->gap_extend;
    ga.xdrop = p->gapped_xdrop;
    ga.cutoff = p->gapped_cutoff;
    ga.smin = INT32_MIN;  // every HSP of each list: this entry point reports raw HSPs
    ga.max_hsps = 0;
    ga.out = reinterpret_cast<DevHsp *>(d_out);
    ga.out_cap = out_capacity;
    ga.cnt = cnt;
    BLAZE_CUDA_TRY(launch_gapped(ga, kBlocks, st, kWarpsPerBlock));
    BLAZE_CUDA_TRY(cudaMemcpyAsync(d_result, &cnt->out_count, sizeof(uint64_t),
                                   cudaMemcpyDeviceToDevice, st));
    BLAZE_CUDA_TRY(cudaMemcpyAsync(d_result + 1, &cnt->flags, sizeof(cnt->flags),
                                   cudaMemcpyDeviceToDevice, st));
    return BLAZE_OK;
}
