// traceback_host.cu -- host side of the traceback stage: items from the last
// run's HSP lists, the kernel launched in passes, and each subject's traced
// HSPs purged, ordered and given final E-values.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handles.h"
#include "internal.h"

// ------------------------------------------------------------------------
// Traceback stage.

// Traces `items` in passes: the first over all of them with many warps and
// small direction buffers, the next ones over those whose alignment did not
// fit, with fewer warps and buffers four times larger. `q`/`qlen` is the
// query of a single-query run; `batch_q`/`batch_qlen` (device arrays) the
// queries of a batched run, indexed by TbItem::query.
static int traceback_passes(blaze_search *s, const std::vector<TbItem> &items, const blaze_params *p,
                            int32_t final_xdrop, const uint8_t *q, int32_t qlen, const uint8_t *const *batch_q,
                            const int32_t *batch_qlen, int32_t max_qlen, std::vector<TbOut> &outs) {
    const blaze_db *db = s->db;
    const size_t n = items.size();
    outs.assign(n, TbOut{});
    s->stats.traceback_ms = 0.f;
    s->stats.traceback_hsps = static_cast<uint32_t>(n);
    s->stats.traceback_cells = 0;
    std::vector<uint32_t> todo(n);
    for (size_t i = 0; i < n; ++i) todo[i] = static_cast<uint32_t>(i);
    unsigned long long cap = s->tb_dir_cap;
    const uint32_t row_cap = static_cast<uint32_t>(max_qlen) + 2u;
    const uint32_t dp_stride = std::max<uint32_t>(db->max_len, 1u) + 2u;
    std::vector<TbItem> pass_items;
    std::vector<TbOut> pass_out;
    int rc;
    for (int attempt = 0; !todo.empty(); ++attempt) {
        if (attempt > 12) return BLAZE_ERR_LIMIT;
        const size_t m = todo.size();
        const int blocks = static_cast<int>(std::min<size_t>(static_cast<size_t>(s->n_sm) * 4,
                                                             (m + kTracebackWarpsPerBlock - 1) / kTracebackWarpsPerBlock));
        const size_t warps = static_cast<size_t>(blocks) * kTracebackWarpsPerBlock;
        pass_items.resize(m);
        for (size_t k = 0; k < m; ++k) pass_items[k] = items[todo[k]];
        pass_out.resize(m);
        if ((rc = s->tb_items.ensure(m)) != BLAZE_OK) return rc;
        if ((rc = s->tb_out.ensure(m)) != BLAZE_OK) return rc;
        if ((rc = s->tb_rows.ensure(warps * 3 * row_cap)) != BLAZE_OK) return rc;
        if ((rc = s->tb_dp.ensure(warps * 2 * dp_stride)) != BLAZE_OK) return rc;
        if ((rc = s->tb_cursor.ensure(1)) != BLAZE_OK) return rc;
        if ((rc = s->tb_dirs.ensure(warps * cap)) != BLAZE_OK) return rc;
        BLAZE_CUDA_TRY(cudaMemcpyAsync(s->tb_items.p, pass_items.data(), sizeof(TbItem) * m, cudaMemcpyHostToDevice,
                                       s->stream));
        s->stats.h2d_bytes += sizeof(TbItem) * m;
        TracebackArgs ta{};
        ta.res = db->d_res;
        ta.off = db->d_off;
        ta.q = q;
        ta.qlen = qlen;
        ta.batch_q = batch_q;
        ta.batch_qlen = batch_qlen;
        ta.items = s->tb_items.p;
        ta.n_items = static_cast<uint32_t>(m);
        ta.out = s->tb_out.p;
        ta.gap_open = p->gap_open;
        ta.gap_extend = p->gap_extend;
        ta.xdrop = final_xdrop;
        ta.dp = s->tb_dp.p;
        ta.dp_stride = dp_stride;
        ta.dirs = s->tb_dirs.p;
        ta.dir_cap = cap;
        ta.rows = s->tb_rows.p;
        ta.row_cap = row_cap;
        ta.cursor = s->tb_cursor.p;
        BLAZE_CUDA_TRY(cudaMemsetAsync(s->tb_cursor.p, 0, sizeof(unsigned long long), s->stream));
        BLAZE_CUDA_TRY(cudaEventRecord(s->ev[1], s->stream));
        BLAZE_CUDA_TRY(launch_traceback(ta, blocks, s->stream));
        BLAZE_CUDA_TRY(cudaEventRecord(s->ev[2], s->stream));
        s->stats.kernel_launches += 1;
        BLAZE_CUDA_TRY(cudaMemcpyAsync(pass_out.data(), s->tb_out.p, sizeof(TbOut) * m, cudaMemcpyDeviceToHost,
                                       s->stream));
        BLAZE_CUDA_TRY(cudaStreamSynchronize(s->stream));
        s->stats.d2h_bytes += sizeof(TbOut) * m;
        float ms = 0.f;
        BLAZE_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev[1], s->ev[2]));
        s->stats.traceback_ms += ms;
        std::vector<uint32_t> again;
        for (size_t k = 0; k < m; ++k) {
            const TbOut &o = pass_out[k];
            s->stats.traceback_cells += static_cast<uint64_t>(o.cells);
            if (o.status == 2) return BLAZE_ERR_INTERNAL;
            if (o.status == 1) again.push_back(todo[k]);
            else outs[todo[k]] = o;
        }
        todo.swap(again);
        cap *= 4;
    }
    return BLAZE_OK;
}

// One subject's traced HSPs: purged of shared start and end points (the
// better kept), ordered as the preliminary stage orders them, given final
// E-values and bit scores and reaped at `evalue`; appended to `out`.
static void traceback_finish_subject(std::vector<TbOut> g, uint32_t oid, const blaze_params &p, double evalue,
                                     std::vector<blaze_aligned_hsp> &out) {
    auto by_start = [](const TbOut &a, const TbOut &b) {
        if (a.q_start != b.q_start) return a.q_start < b.q_start;
        if (a.s_start != b.s_start) return a.s_start < b.s_start;
        if (a.score != b.score) return a.score > b.score;
        if (a.q_end != b.q_end) return a.q_end > b.q_end;
        return a.s_end > b.s_end;
    };
    auto by_end = [](const TbOut &a, const TbOut &b) {
        if (a.q_end != b.q_end) return a.q_end < b.q_end;
        if (a.s_end != b.s_end) return a.s_end < b.s_end;
        if (a.score != b.score) return a.score > b.score;
        if (a.q_start != b.q_start) return a.q_start < b.q_start;
        return a.s_start < b.s_start;
    };
    auto by_score = [](const TbOut &a, const TbOut &b) {
        if (a.score != b.score) return a.score > b.score;
        if (a.s_start != b.s_start) return a.s_start < b.s_start;
        if (a.s_end != b.s_end) return a.s_end > b.s_end;
        if (a.q_start != b.q_start) return a.q_start < b.q_start;
        return a.q_end > b.q_end;
    };
    std::stable_sort(g.begin(), g.end(), by_start);
    std::vector<TbOut> m;
    for (const TbOut &o : g)
        if (m.empty() || o.q_start != m.back().q_start || o.s_start != m.back().s_start) m.push_back(o);
    std::stable_sort(m.begin(), m.end(), by_end);
    std::vector<TbOut> m2;
    for (const TbOut &o : m)
        if (m2.empty() || o.q_end != m2.back().q_end || o.s_end != m2.back().s_end) m2.push_back(o);
    std::stable_sort(m2.begin(), m2.end(), by_score);
    const double ln2 = std::log(2.0), lnK = std::log(p.K);
    for (const TbOut &o : m2) {
        blaze_aligned_hsp h{};
        h.oid = oid;
        h.score = o.score;
        h.q_start = o.q_start;
        h.q_end = o.q_end;
        h.s_start = o.s_start;
        h.s_end = o.s_end;
        h.length = o.length;
        h.identities = o.identities;
        h.positives = o.positives;
        h.mismatches = o.mismatches;
        h.gap_opens = o.gap_opens;
        h.gaps = o.gaps;
        h.evalue = p.eff_searchsp * p.K * std::exp(-p.lambda * static_cast<double>(o.score));
        h.bit_score = (p.lambda * static_cast<double>(o.score) - lnK) / ln2;
        if (h.evalue <= evalue) out.push_back(h);
    }
}

static int tb_item(const blaze_db *db, const blaze_hsp &h, int32_t qlen, uint32_t query, TbItem *it) {
    if (h.oid >= db->n || h.q_gapped_start < 0 || h.q_gapped_start >= qlen) return BLAZE_ERR_INVALID_ARG;
    const uint32_t sub = db->sorted_of[h.oid];
    if (h.s_gapped_start < 0 || static_cast<uint64_t>(h.s_gapped_start) >= db->h_off[sub + 1] - db->h_off[sub])
        return BLAZE_ERR_INVALID_ARG;
    *it = TbItem{sub, h.q_gapped_start, h.s_gapped_start, query};
    return BLAZE_OK;
}

extern "C" int blaze_search_traceback(blaze_search *s, const blaze_query *q, const blaze_params *p,
                                      int32_t final_xdrop, double evalue, uint64_t *n_hsps) try {
    if (!s || !q || !p || final_xdrop <= 0 || q->device != s->db->device || s->last_batched)
        return BLAZE_ERR_INVALID_ARG;
    int rc = check_params(p);
    if (rc != BLAZE_OK) return rc;
    if (n_hsps) *n_hsps = 0;
    s->tb_results.clear();
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    const size_t n = s->results.size();
    std::vector<TbItem> items(n);
    for (size_t i = 0; i < n; ++i)
        if ((rc = tb_item(s->db, s->results[i], q->qlen, 0u, &items[i])) != BLAZE_OK) return rc;
    std::vector<TbOut> outs;
    if ((rc = traceback_passes(s, items, p, final_xdrop, q->d_q, q->qlen, nullptr, nullptr, q->qlen, outs)) !=
        BLAZE_OK)
        return rc;
    for (size_t i = 0; i < n;) {
        size_t j = i;
        while (j < n && s->results[j].oid == s->results[i].oid) ++j;
        traceback_finish_subject(std::vector<TbOut>(outs.begin() + i, outs.begin() + j), s->results[i].oid, *p,
                                 evalue, s->tb_results);
        i = j;
    }
    if (n_hsps) *n_hsps = s->tb_results.size();
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_traceback_batch(blaze_search *s, const blaze_batch *b, const blaze_params *params,
                                            int32_t final_xdrop, double evalue, uint64_t *n_hsps) try {
    if (!s || !b || !params || final_xdrop <= 0 || !s->last_batched || s->last_batch != b)
        return BLAZE_ERR_INVALID_ARG;
    int rc;
    for (uint32_t i = 0; i < b->n; ++i)
        if ((rc = check_params(&params[i])) != BLAZE_OK) return rc;
    if (n_hsps) *n_hsps = 0;
    s->tb_batch_results.clear();
    BLAZE_CUDA_TRY(cudaSetDevice(s->db->device));
    const size_t n = s->batch_results.size();
    std::vector<TbItem> items(n);
    int32_t max_qlen = 1;
    for (uint32_t i = 0; i < b->n; ++i) max_qlen = std::max(max_qlen, b->qlen[i]);
    for (size_t i = 0; i < n; ++i) {
        const blaze_batch_hsp &bh = s->batch_results[i];
        if (bh.query >= b->n) return BLAZE_ERR_INVALID_ARG;
        if ((rc = tb_item(s->db, bh.hsp, b->qlen[bh.query], bh.query, &items[i])) != BLAZE_OK) return rc;
    }
    // the per-query arrays of the last batched run (batch order) are still
    // on the device
    std::vector<TbOut> outs;
    if ((rc = traceback_passes(s, items, &params[0], final_xdrop, nullptr, 0, s->bqptr.p, s->bqlen.p, max_qlen,
                               outs)) != BLAZE_OK)
        return rc;
    std::vector<blaze_aligned_hsp> one;
    for (size_t i = 0; i < n;) {
        size_t j = i;
        const uint32_t qi = s->batch_results[i].query, oid = s->batch_results[i].hsp.oid;
        while (j < n && s->batch_results[j].query == qi && s->batch_results[j].hsp.oid == oid) ++j;
        one.clear();
        traceback_finish_subject(std::vector<TbOut>(outs.begin() + i, outs.begin() + j), oid, params[qi], evalue,
                                 one);
        for (const blaze_aligned_hsp &h : one) s->tb_batch_results.push_back(blaze_batch_aligned_hsp{qi, 0u, h});
        i = j;
    }
    if (n_hsps) *n_hsps = s->tb_batch_results.size();
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_search_traceback_batch_results(const blaze_search *s, blaze_batch_aligned_hsp *out,
                                                    uint64_t capacity, uint64_t *n_hsps) {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    const size_t n = s->tb_batch_results.size();
    if (n_hsps) *n_hsps = n;
    if (capacity < n) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (n && !out) return BLAZE_ERR_INVALID_ARG;
    if (n) std::memcpy(out, s->tb_batch_results.data(), sizeof(blaze_batch_aligned_hsp) * n);
    return BLAZE_OK;
}

extern "C" int blaze_search_traceback_results(const blaze_search *s, blaze_aligned_hsp *out, uint64_t capacity,
                                              uint64_t *n_hsps) {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    const size_t n = s->tb_results.size();
    if (n_hsps) *n_hsps = n;
    if (capacity < n) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (n && !out) return BLAZE_ERR_INVALID_ARG;
    if (n) std::memcpy(out, s->tb_results.data(), sizeof(blaze_aligned_hsp) * n);
    return BLAZE_OK;
}
