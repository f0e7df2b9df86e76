// seqsrc.cpp -- the resident database built from a BlastSeqSrc-shaped source
// (blaze_db_create_from_source).
//
// The reference's GPU driver gathers subjects chunk by chunk through
// BlastSeqSrcGetSequence into pinned buffers and copies each whole buffer to
// the device for every query (BLAZE_gpu/gpuBLAZE.cu:1587-1618). Here the
// source is read once: lengths first (GetSeqLen, or one fetch pass), then the
// sequences in ascending length order through two pinned staging buffers
// whose copies to the device overlap the next buffer's gather, straight into
// the length-sorted resident layout blaze_db_create builds -- no second host
// copy of the database.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "handles.h"
#include "internal.h"

namespace {

constexpr size_t kStageBytes = 32u << 20;  // per pinned staging buffer

// Fills two pinned buffers in turn and copies each, once full, to the next
// bytes of `dst` on `st`; a buffer is refilled only after its copy is done.
class Uploader {
  public:
    Uploader(uint8_t *dst, cudaStream_t st) : dst_(dst), st_(st) {}
    ~Uploader() {
        for (int i = 0; i < 2; ++i) {
            if (ev_[i]) {
                cudaEventSynchronize(ev_[i]);
                cudaEventDestroy(ev_[i]);
            }
            if (buf_[i]) cudaFreeHost(buf_[i]);
        }
    }
    int init() {
        for (int i = 0; i < 2; ++i) {
            BLAZE_CUDA_TRY(cudaMallocHost(&buf_[i], kStageBytes));
            BLAZE_CUDA_TRY(cudaEventCreateWithFlags(&ev_[i], cudaEventDisableTiming));
        }
        return BLAZE_OK;
    }
    int put(const uint8_t *p, size_t n) {
        while (n > 0) {
            const size_t k = std::min(n, kStageBytes - fill_);
            std::memcpy(buf_[cur_] + fill_, p, k);
            fill_ += k;
            p += k;
            n -= k;
            if (fill_ == kStageBytes) {
                int rc = flush();
                if (rc != BLAZE_OK) return rc;
            }
        }
        return BLAZE_OK;
    }
    int flush() {
        if (fill_ == 0) return BLAZE_OK;
        BLAZE_CUDA_TRY(cudaMemcpyAsync(dst_ + done_, buf_[cur_], fill_, cudaMemcpyHostToDevice, st_));
        BLAZE_CUDA_TRY(cudaEventRecord(ev_[cur_], st_));
        pending_[cur_] = true;
        done_ += fill_;
        fill_ = 0;
        cur_ ^= 1;
        if (pending_[cur_]) {
            BLAZE_CUDA_TRY(cudaEventSynchronize(ev_[cur_]));
            pending_[cur_] = false;
        }
        return BLAZE_OK;
    }
    int finish() {
        int rc = flush();
        if (rc != BLAZE_OK) return rc;
        BLAZE_CUDA_TRY(cudaStreamSynchronize(st_));
        pending_[0] = pending_[1] = false;
        return BLAZE_OK;
    }

  private:
    uint8_t *dst_;
    cudaStream_t st_;
    uint8_t *buf_[2] = {nullptr, nullptr};
    cudaEvent_t ev_[2] = {nullptr, nullptr};
    bool pending_[2] = {false, false};
    int cur_ = 0;
    size_t fill_ = 0;
    uint64_t done_ = 0;
};

// get_sequence + checks + release_sequence; *len_out is the returned length.
int fetch(const blaze_seq_source *src, uint32_t oid, const uint8_t **res, uint32_t *len_out) {
    *res = nullptr;
    *len_out = 0;
    if (src->get_sequence(src->user, oid, res, len_out) != 0) return BLAZE_ERR_INVALID_ARG;
    if (*len_out > 0 && !*res) return BLAZE_ERR_INVALID_ARG;
    return BLAZE_OK;
}

void release(const blaze_seq_source *src, uint32_t oid) {
    if (src->release_sequence) src->release_sequence(src->user, oid);
}

}  // namespace

extern "C" int blaze_db_create_from_source(int device, const blaze_seq_source *src, blaze_db **out) try {
    if (!out || !src || !src->get_num_seqs || !src->get_sequence) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    blaze_device_count(&ndev);
    if (ndev == 0) return BLAZE_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return BLAZE_ERR_INVALID_ARG;
    const int64_t n64 = src->get_num_seqs(src->user);
    if (n64 < 0) return BLAZE_ERR_INVALID_ARG;
    if (n64 >= static_cast<int64_t>(UINT32_MAX)) return BLAZE_ERR_LIMIT;
    const uint32_t n = static_cast<uint32_t>(n64);

    // the OIDs to search (BlastSeqSrcIteratorNext), each at most once
    std::vector<uint8_t> included(n, src->iter_next ? 0 : 1);
    if (src->iter_next) {
        for (uint64_t visits = 0;; ++visits) {
            const int64_t oid = src->iter_next(src->user);
            if (oid < 0) break;
            if (oid >= n64 || included[oid] || visits >= n) return BLAZE_ERR_INVALID_ARG;
            included[oid] = 1;
        }
    }

    // lengths (BlastSeqSrcGetSeqLen, or one fetch pass)
    std::vector<uint64_t> len(n, 0);
    uint64_t total = 0, longest = 0;
    for (uint32_t oid = 0; oid < n; ++oid) {
        if (!included[oid]) continue;
        int64_t L = 0;
        if (src->get_seq_len) {
            L = src->get_seq_len(src->user, oid);
        } else {
            const uint8_t *r = nullptr;
            uint32_t l32 = 0;
            int rc = fetch(src, oid, &r, &l32);
            release(src, oid);
            if (rc != BLAZE_OK) return rc;
            L = l32;
        }
        if (L < 0) return BLAZE_ERR_INVALID_ARG;
        if (static_cast<uint64_t>(L) > kMaxSubjectLength) return BLAZE_ERR_LIMIT;
        len[oid] = static_cast<uint64_t>(L);
        total += len[oid];
        longest = std::max(longest, len[oid]);
    }
    // the source's own totals, when it reports them, cover every OID
    if (!src->iter_next) {
        if (src->get_tot_len && src->get_tot_len(src->user) != static_cast<int64_t>(total))
            return BLAZE_ERR_INVALID_ARG;
        if (src->get_max_seq_len && src->get_max_seq_len(src->user) != static_cast<int64_t>(longest))
            return BLAZE_ERR_INVALID_ARG;
    }

    // length-sorted order (stable: equal lengths keep OID order)
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return len[a] < len[b]; });
    std::vector<uint64_t> off(static_cast<size_t>(n) + 1, 0);
    for (uint32_t k = 0; k < n; ++k) off[k + 1] = off[k] + len[order[k]];

    BLAZE_CUDA_TRY(cudaSetDevice(device));
    auto *db = new blaze_db();
    db->device = device;
    db->n = n;
    db->total = total;
    db->max_len = static_cast<uint32_t>(longest);
    db->oid_of = order;
    db->sorted_of.resize(n);
    for (uint32_t k = 0; k < n; ++k) db->sorted_of[order[k]] = k;
    cudaStream_t st = nullptr;
    int rc = BLAZE_OK;
    do {
        cudaError_t e = cudaMalloc(&db->d_res, total + 64);
        if (e == cudaSuccess) e = cudaMalloc(&db->d_off, sizeof(uint64_t) * (static_cast<size_t>(n) + 1));
        if (e == cudaSuccess) e = cudaMalloc(&db->d_oid, sizeof(uint32_t) * std::max<uint32_t>(n, 1));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            last_cuda_error(e);
            rc = e == cudaErrorMemoryAllocation ? BLAZE_ERR_OUT_OF_MEMORY : BLAZE_ERR_CUDA;
            break;
        }
        Uploader up(db->d_res, st);
        if ((rc = up.init()) != BLAZE_OK) break;
        for (uint32_t k = 0; k < n && rc == BLAZE_OK; ++k) {
            const uint32_t oid = order[k];
            if (len[oid] == 0) continue;
            const uint8_t *r = nullptr;
            uint32_t l32 = 0;
            rc = fetch(src, oid, &r, &l32);
            if (rc == BLAZE_OK && (l32 != len[oid] || !valid_residues(r, l32))) rc = BLAZE_ERR_INVALID_ARG;
            if (rc == BLAZE_OK) rc = up.put(r, l32);
            release(src, oid);
        }
        if (rc == BLAZE_OK) rc = up.finish();
        if (rc != BLAZE_OK) break;
        e = cudaMemset(db->d_res + total, 0, 64);
        if (e == cudaSuccess)
            e = cudaMemcpy(db->d_off, off.data(), sizeof(uint64_t) * (static_cast<size_t>(n) + 1),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess && n) e = cudaMemcpy(db->d_oid, order.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            last_cuda_error(e);
            rc = BLAZE_ERR_CUDA;
        }
    } while (false);
    if (st) cudaStreamDestroy(st);
    if (rc != BLAZE_OK) {
        blaze_db_free(db);
        return rc;
    }
    db->h_off.swap(off);
    *out = db;
    return BLAZE_OK;
} BLAZE_ABI_CATCH
