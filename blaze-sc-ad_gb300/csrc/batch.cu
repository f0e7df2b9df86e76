// batch.cu -- query batches of the batched form: every query's word tables
// built on the host and uploaded into one set of device arrays (refilled in
// place by the serving loop).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "handles.h"
#include "internal.h"

static int check_batch_input(const uint8_t *residues, const uint64_t *offsets, uint32_t n_queries) {
    if (!residues || !offsets || n_queries == 0) return BLAZE_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n_queries; ++i) {
        if (offsets[i + 1] <= offsets[i]) return BLAZE_ERR_INVALID_ARG;
        if (offsets[i + 1] - offsets[i] > static_cast<uint64_t>(kMaxQueryLength)) return BLAZE_ERR_LIMIT;
        if (!valid_residues(residues + offsets[i], offsets[i + 1] - offsets[i])) return BLAZE_ERR_INVALID_ARG;
    }
    return BLAZE_OK;
}

// Builds the word tables of every query on the host and uploads them into
// the batch's device buffers, growing those only when they are too small
// (so that a refilled batch allocates nothing once it has seen its largest
// load). Copies go on `stream` (0: synchronous).
static int batch_fill(blaze_batch *b, const uint8_t *residues, const uint64_t *offsets, uint32_t n_queries,
                      int32_t word_threshold, cudaStream_t stream) {
    b->n = n_queries;
    b->threshold = word_threshold;
    b->qlen.clear();
    b->res_off.clear();
    b->off_off.clear();
    std::vector<uint8_t> res;
    std::vector<uint32_t> cs_all(static_cast<size_t>(n_queries) * (kWords + 1));
    std::vector<uint32_t> pack_all(static_cast<size_t>(n_queries) * kWords);
    std::vector<uint32_t> pres_all(static_cast<size_t>(n_queries) * kPresenceWords, 0u);
    std::vector<uint16_t> offs_all;
    for (uint32_t i = 0; i < n_queries; ++i) {
        const int32_t len = static_cast<int32_t>(offsets[i + 1] - offsets[i]);
        const uint8_t *q = residues + offsets[i];
        b->qlen.push_back(len);
        b->res_off.push_back(res.size());
        res.insert(res.end(), q, q + len);
        res.resize((res.size() + 63) & ~static_cast<size_t>(63), 0);  // 64-byte separation
        uint32_t *cs = cs_all.data() + static_cast<size_t>(i) * (kWords + 1);
        uint16_t *offs = nullptr;
        uint32_t n_off = 0;
        int rc = build_lookup(q, len, word_threshold, cs, &offs, &n_off);
        if (rc != BLAZE_OK) return rc;
        b->off_off.push_back(offs_all.size());
        offs_all.insert(offs_all.end(), offs, offs + n_off);
        std::free(offs);
        pack_word_cells(cs, pack_all.data() + static_cast<size_t>(i) * kWords,
                        pres_all.data() + static_cast<size_t>(i) * kPresenceWords);
    }
    res.resize(res.size() + 64, 0);
    if (offs_all.empty()) offs_all.push_back(0);
    // a refill grows by half again so that slowly rising loads settle
    const size_t slack = stream ? 2 : 1;
    auto grow = [&](auto &buf, size_t want) {
        return want <= buf.n ? BLAZE_OK : buf.ensure(want + (slack - 1) * want / 2);
    };
    int rc = grow(b->res, res.size());
    if (rc == BLAZE_OK) rc = grow(b->cell_start, cs_all.size());
    if (rc == BLAZE_OK) rc = grow(b->cell_pack, pack_all.size());
    if (rc == BLAZE_OK) rc = grow(b->presence, pres_all.size());
    if (rc == BLAZE_OK) rc = grow(b->cell_off, offs_all.size());
    if (rc != BLAZE_OK) return rc;
    b->d_res = b->res.p;
    b->d_cell_start = b->cell_start.p;
    b->d_cell_pack = b->cell_pack.p;
    b->d_presence = b->presence.p;
    b->d_cell_off = b->cell_off.p;
    auto put = [&](void *dst, const void *src, size_t bytes) {
        return stream ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream)
                      : cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    cudaError_t e = put(b->d_res, res.data(), res.size());
    if (e == cudaSuccess) e = put(b->d_cell_start, cs_all.data(), sizeof(uint32_t) * cs_all.size());
    if (e == cudaSuccess) e = put(b->d_cell_pack, pack_all.data(), sizeof(uint32_t) * pack_all.size());
    if (e == cudaSuccess) e = put(b->d_presence, pres_all.data(), sizeof(uint32_t) * pres_all.size());
    if (e == cudaSuccess) e = put(b->d_cell_off, offs_all.data(), sizeof(uint16_t) * offs_all.size());
    // the host arrays die with this frame: the copies must have read them
    if (e == cudaSuccess && stream) e = cudaStreamSynchronize(stream);
    b->upload_bytes = res.size() + sizeof(uint32_t) * (cs_all.size() + pack_all.size() + pres_all.size()) +
                      sizeof(uint16_t) * offs_all.size();
    b->device_bytes = b->res.n + sizeof(uint32_t) * (b->cell_start.n + b->cell_pack.n + b->presence.n) +
                      sizeof(uint16_t) * b->cell_off.n;
    if (e != cudaSuccess) {
        last_cuda_error(e);
        return e == cudaErrorMemoryAllocation ? BLAZE_ERR_OUT_OF_MEMORY : BLAZE_ERR_CUDA;
    }
    return BLAZE_OK;
}

extern "C" int blaze_batch_create(const blaze_db *db, const uint8_t *residues, const uint64_t *offsets,
                                  uint32_t n_queries, int32_t word_threshold, blaze_batch **out) try {
    if (!db || !out) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    const int vrc = check_batch_input(residues, offsets, n_queries);
    if (vrc != BLAZE_OK) return vrc;
    BLAZE_CUDA_TRY(cudaSetDevice(db->device));
    auto *b = new blaze_batch();
    b->device = db->device;
    const int rc = batch_fill(b, residues, offsets, n_queries, word_threshold, nullptr);
    if (rc != BLAZE_OK) {
        blaze_batch_free(b);
        return rc;
    }
    *out = b;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

int batch_refill(blaze_search *s, blaze_batch **inout, const uint8_t *residues, const uint64_t *offsets,
                 uint32_t n_queries, int32_t word_threshold) {
    if (!s || !inout) return BLAZE_ERR_INVALID_ARG;
    const int vrc = check_batch_input(residues, offsets, n_queries);
    if (vrc != BLAZE_OK) return vrc;
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    if (!*inout) {
        *inout = new blaze_batch();
        (*inout)->device = s->db->device;
    }
    return batch_fill(*inout, residues, offsets, n_queries, word_threshold, s->stream);
}

extern "C" int blaze_batch_free(blaze_batch *b) {
    if (!b) return BLAZE_OK;
    cudaSetDevice(b->device);
    b->res.release();
    b->cell_start.release();
    b->cell_pack.release();
    b->presence.release();
    b->cell_off.release();
    delete b;
    return BLAZE_OK;
}

extern "C" int blaze_batch_info(const blaze_batch *b, uint32_t *n_queries, uint64_t *device_bytes) {
    if (!b) return BLAZE_ERR_INVALID_ARG;
    if (n_queries) *n_queries = b->n;
    if (device_bytes) *device_bytes = b->device_bytes;
    return BLAZE_OK;
}
