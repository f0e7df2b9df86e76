// server.cpp -- the serving loop of libblaze103: continuous batching of
// arriving queries over the resident database (C++ threads above the C ABI).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "blaze_prelim.h"
#include "internal.h"

namespace {

using Clock = std::chrono::steady_clock;

// Device bytes a query adds to a batch beyond its word tables: seed, init-hit
// and HSP buffers scale with the work a query brings, a few hundred bytes per
// residue on these shapes, plus a fixed part.
constexpr uint64_t kPerQueryFixed = 1u << 20;
constexpr uint64_t kPerResidue = 512;
constexpr uint64_t kTableBytes = 4ull * (2 * 21952 + 1 + 686);
constexpr uint32_t kMaxSlots = 64;  // worker threads (each with its search context)
// From this many database residues on, a batched run launches the word
// finder once per query (a query alone fills the GPU) and batching saves
// nothing on the device: batches are then kept small so that each query's
// results return soon, and the workers' GPU work runs one batch at a time
// (their host work -- lookup tables, uploads, results -- still overlaps), since
// concurrent whole-GPU launches only contend.
constexpr uint64_t kLargeDbResidues = 1ull << 27;
constexpr uint32_t kLargeDbBatch = 4;

struct Request {
    uint64_t ticket;
    std::vector<uint8_t> residues;
    Clock::time_point submitted;
    uint64_t estimate;
};

struct Result {
    bool done = false;
    int status = BLAZE_OK;
    int cuda_error = 0;  // the worker's CUDA error when status is BLAZE_ERR_CUDA
    std::vector<blaze_hsp> hsps;
    double latency_ms = 0;
};

}  // namespace

struct blaze_server {
    blaze_db *db = nullptr;
    blaze_server_config cfg{};
    uint64_t db_residues = 0;
    uint32_t db_subjects = 0;
    std::mutex mu;
    std::condition_variable queue_cv, done_cv;
    std::deque<Request> queue;
    std::unordered_map<uint64_t, Result> results;
    uint64_t next_ticket = 1;
    uint64_t in_flight_bytes = 0;
    bool stopping = false;
    bool one_gpu_batch = false;  // large database: see kLargeDbResidues
    uint32_t max_batch = 1;      // the configured cap, or kLargeDbBatch on a large database
    std::mutex gpu_mu;
    std::vector<std::thread> workers;
    // statistics
    uint64_t submitted = 0, completed = 0, batches = 0, residues = 0;
    std::vector<double> latencies;
    bool any_submit = false;
    Clock::time_point first_submit, last_done;
};

namespace {

uint64_t estimate_bytes(int32_t len) { return kPerQueryFixed + kTableBytes + kPerResidue * static_cast<uint64_t>(len); }

// Takes the next batch: waits for a first query, then up to batch_window_us
// for more, admitting while the memory budget allows. Returns false on stop.
bool take_batch(blaze_server *s, std::vector<Request> &batch, uint64_t &bytes) {
    std::unique_lock<std::mutex> lk(s->mu);
    batch.clear();
    bytes = 0;
    for (;;) {
        s->queue_cv.wait(lk, [&] { return s->stopping || !s->queue.empty(); });
        if (s->queue.empty()) return false;  // stopping with nothing left
        const uint64_t budget = s->cfg.memory_budget;
        const uint64_t first = s->queue.front().estimate;
        // the first query waits until it fits next to the batches in flight
        // (alone it always fits: an empty device takes any single query)
        if (budget && s->in_flight_bytes > 0 && s->in_flight_bytes + first > budget) {
            s->done_cv.wait(lk);
            continue;
        }
        break;
    }
    const auto deadline = Clock::now() + std::chrono::microseconds(s->cfg.batch_window_us);
    for (;;) {
        while (!s->queue.empty() && batch.size() < s->max_batch) {
            const uint64_t est = s->queue.front().estimate;
            const uint64_t budget = s->cfg.memory_budget;
            if (!batch.empty() && budget && s->in_flight_bytes + bytes + est > budget) break;
            bytes += est;
            batch.push_back(std::move(s->queue.front()));
            s->queue.pop_front();
        }
        if (batch.size() >= s->max_batch || s->stopping) break;
        if (s->queue_cv.wait_until(lk, deadline) == std::cv_status::timeout) {
            // take whatever arrived in the last instant
            while (!s->queue.empty() && batch.size() < s->max_batch) {
                const uint64_t est = s->queue.front().estimate;
                if (s->cfg.memory_budget && s->in_flight_bytes + bytes + est > s->cfg.memory_budget) break;
                bytes += est;
                batch.push_back(std::move(s->queue.front()));
                s->queue.pop_front();
            }
            break;
        }
    }
    s->in_flight_bytes += bytes;
    return true;
}

void worker(blaze_server *s) {
    blaze_search *search = nullptr;
    int create_rc = blaze_search_create(s->db, &search);
    const blaze_tuning &t = s->cfg.tuning;
    if (create_rc == BLAZE_OK && (t.stage_bytes | t.tile_residues | t.max_warps_per_block | t.launch_mode))
        create_rc = blaze_search_set_tuning(search, &t);
    blaze_batch *b = nullptr;  // refilled for every batch: no allocation once warm
    std::vector<Request> batch;
    std::vector<blaze_batch_hsp> out;
    uint64_t bytes = 0;
    while (take_batch(s, batch, bytes)) {
        const size_t n = batch.size();
        uint64_t batch_residues = 0;
        int rc = create_rc;
        uint64_t n_hsps = 0;
        try {  // a failed host allocation fails this batch, not the process
            std::vector<uint8_t> res;
            std::vector<uint64_t> off(n + 1, 0);
            std::vector<blaze_params> params(n);
            for (size_t i = 0; i < n; ++i) {
                res.insert(res.end(), batch[i].residues.begin(), batch[i].residues.end());
                off[i + 1] = res.size();
                blaze_params_default(static_cast<int32_t>(batch[i].residues.size()), s->db_residues,
                                     s->db_subjects, s->cfg.evalue, &params[i]);
                batch_residues += s->db_residues;
            }
            if (rc == BLAZE_OK) rc = batch_refill(search, &b, res.data(), off.data(), static_cast<uint32_t>(n), 11);
            if (rc == BLAZE_OK) {
                std::unique_lock<std::mutex> gpu(s->gpu_mu, std::defer_lock);
                if (s->one_gpu_batch) gpu.lock();
                rc = blaze_search_run_batch(search, b, params.data(), &n_hsps);
            }
            if (rc == BLAZE_OK) {
                out.resize(n_hsps);
                rc = blaze_search_batch_results(search, out.data(), n_hsps, &n_hsps);
            }
        } catch (const std::bad_alloc &) {
            rc = BLAZE_ERR_OUT_OF_MEMORY;
        }
        const auto now = Clock::now();
        const int cuda_error = rc == BLAZE_ERR_CUDA ? last_cuda_error_code() : 0;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            size_t k = 0;
            for (size_t i = 0; i < n; ++i) {
                Result &r = s->results[batch[i].ticket];
                r.status = rc;
                r.cuda_error = cuda_error;
                r.hsps.clear();
                while (rc == BLAZE_OK && k < n_hsps && out[k].query == i) r.hsps.push_back(out[k++].hsp);
                r.latency_ms = std::chrono::duration<double, std::milli>(now - batch[i].submitted).count();
                r.done = true;
                s->latencies.push_back(r.latency_ms);
            }
            s->completed += n;
            s->batches += 1;
            s->residues += batch_residues;
            s->last_done = now;
            s->in_flight_bytes -= bytes;
        }
        s->done_cv.notify_all();
        s->queue_cv.notify_all();
    }
    blaze_batch_free(b);
    if (search) blaze_search_free(search);
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * static_cast<double>(v.size() - 1);
    const size_t lo = static_cast<size_t>(pos);
    const size_t hi = std::min(lo + 1, v.size() - 1);
    return v[lo] + (v[hi] - v[lo]) * (pos - static_cast<double>(lo));
}

}  // namespace

extern "C" int blaze_server_create(blaze_db *db, const blaze_server_config *cfg, blaze_server **out) try {
    if (!db || !cfg || !out || cfg->slots == 0 || cfg->max_batch == 0 || cfg->evalue <= 0) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->slots > kMaxSlots) return BLAZE_ERR_LIMIT;
    auto *s = new blaze_server();
    s->db = db;
    s->cfg = *cfg;
    uint32_t max_len = 0;
    blaze_db_info(db, &s->db_residues, &s->db_subjects, &max_len);
    s->one_gpu_batch = s->db_residues >= kLargeDbResidues && cfg->tuning.batch_launch != 1;
    s->max_batch = s->one_gpu_batch ? std::min(cfg->max_batch, kLargeDbBatch) : cfg->max_batch;
    try {
        for (uint32_t i = 0; i < cfg->slots; ++i) s->workers.emplace_back(worker, s);
    } catch (...) {  // a thread that would not start: stop the ones that did
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stopping = true;
        }
        s->queue_cv.notify_all();
        for (std::thread &t : s->workers) t.join();
        delete s;
        return BLAZE_ERR_INTERNAL;
    }
    *out = s;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_server_submit(blaze_server *s, const uint8_t *query, int32_t length, uint64_t *ticket) try {
    if (!s || !query || length <= 0 || !ticket) return BLAZE_ERR_INVALID_ARG;
    if (length > 32000) return BLAZE_ERR_LIMIT;
    for (int32_t i = 0; i < length; ++i)
        if (query[i] == 0 || query[i] >= 28) return BLAZE_ERR_INVALID_ARG;
    Request r;
    r.residues.assign(query, query + length);
    r.submitted = Clock::now();
    r.estimate = estimate_bytes(length);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) return BLAZE_ERR_INVALID_ARG;
        r.ticket = s->next_ticket++;
        *ticket = r.ticket;
        s->results[r.ticket];  // registered, not done
        if (!s->any_submit) {
            s->any_submit = true;
            s->first_submit = r.submitted;
        }
        ++s->submitted;
        s->queue.push_back(std::move(r));
    }
    s->queue_cv.notify_one();
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_server_wait(blaze_server *s, uint64_t ticket, int32_t timeout_ms, uint64_t *n_hsps) try {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->results.find(ticket);
    if (it == s->results.end()) return BLAZE_ERR_INVALID_ARG;
    auto ready = [&] { return s->results[ticket].done; };
    if (timeout_ms < 0) {
        s->done_cv.wait(lk, ready);
    } else if (!s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return BLAZE_ERR_LIMIT;
    }
    const Result &r = s->results[ticket];
    if (n_hsps) *n_hsps = r.hsps.size();
    if (r.status == BLAZE_ERR_CUDA) set_last_cuda_error_code(r.cuda_error);
    return r.status;
} BLAZE_ABI_CATCH

extern "C" int blaze_server_take(blaze_server *s, uint64_t ticket, blaze_hsp *out, uint64_t capacity,
                                 uint64_t *n_hsps, double *latency_ms) try {
    if (!s) return BLAZE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->results.find(ticket);
    if (it == s->results.end() || !it->second.done) return BLAZE_ERR_INVALID_ARG;
    const Result &r = it->second;
    if (n_hsps) *n_hsps = r.hsps.size();
    if (latency_ms) *latency_ms = r.latency_ms;
    if (r.status != BLAZE_OK) {
        const int st = r.status;
        if (st == BLAZE_ERR_CUDA) set_last_cuda_error_code(r.cuda_error);
        s->results.erase(it);
        return st;
    }
    if (capacity < r.hsps.size()) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (!r.hsps.empty()) {
        if (!out) return BLAZE_ERR_INVALID_ARG;
        std::memcpy(out, r.hsps.data(), sizeof(blaze_hsp) * r.hsps.size());
    }
    s->results.erase(it);
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_server_stats_get(blaze_server *s, blaze_server_stats *out) try {
    if (!s || !out) return BLAZE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->batches = s->batches;
    out->residues = s->residues;
    out->latency_p50_ms = percentile(s->latencies, 0.50);
    out->latency_p99_ms = percentile(s->latencies, 0.99);
    out->latency_max_ms = s->latencies.empty() ? 0.0 : *std::max_element(s->latencies.begin(), s->latencies.end());
    if (s->any_submit && s->completed)
        out->busy_s = std::chrono::duration<double>(s->last_done - s->first_submit).count();
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_server_free(blaze_server *s) {
    if (!s) return BLAZE_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->queue_cv.notify_all();
    s->done_cv.notify_all();
    for (std::thread &t : s->workers) t.join();
    delete s;
    return BLAZE_OK;
}
