// host.cpp -- host-side pieces of libblaze103 that need no GPU: the BLOSUM62
// table, the query word lookup and the NCBI-default search parameters.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace blaze {

const int32_t kBlosum62[kAlphabet][kAlphabet] = {
#include "blosum62.inc"
};

namespace {

// Neighbourhood of every three-letter word for one threshold, in CSR form:
// words v with score(w, v) >= threshold, plus w itself
// (BLAZE_ncbi/prelim_stage.cpp:135-155 enumerates the same set; :378-383
// keeps the exact word). Computed once per threshold and cached.
struct Neighbourhood {
    std::vector<uint32_t> start;  // kWords + 1
    std::vector<uint16_t> words;  // word index < 21952 fits 16 bits
};

std::mutex g_nb_mutex;
std::map<int32_t, Neighbourhood *> g_nb_cache;

const Neighbourhood *neighbourhood(int32_t threshold) {
    std::lock_guard<std::mutex> lock(g_nb_mutex);
    auto it = g_nb_cache.find(threshold);
    if (it != g_nb_cache.end()) return it->second;
    auto *nb = new Neighbourhood();
    nb->start.resize(kWords + 1);
    int32_t row_max[kAlphabet];
    for (int a = 0; a < kAlphabet; ++a)
        row_max[a] = *std::max_element(kBlosum62[a], kBlosum62[a] + kAlphabet);
    for (int w = 0; w < kWords; ++w) {
        nb->start[w] = static_cast<uint32_t>(nb->words.size());
        const int x = w / 784, y = (w / 28) % 28, z = w % 28;
        bool self_added = false;
        for (int a = 0; a < kAlphabet; ++a) {
            const int32_t s0 = kBlosum62[x][a];
            if (s0 + row_max[y] + row_max[z] < threshold) continue;
            for (int b = 0; b < kAlphabet; ++b) {
                const int32_t s1 = s0 + kBlosum62[y][b];
                if (s1 + row_max[z] < threshold) continue;
                for (int c = 0; c < kAlphabet; ++c) {
                    if (s1 + kBlosum62[z][c] >= threshold) {
                        const int v = a * 784 + b * 28 + c;
                        nb->words.push_back(static_cast<uint16_t>(v));
                        if (v == w) self_added = true;
                    }
                }
            }
        }
        if (!self_added) {
            // keep cells sorted by word index: insert w at its place
            auto first = nb->words.begin() + nb->start[w];
            nb->words.insert(std::upper_bound(first, nb->words.end(), static_cast<uint16_t>(w)),
                             static_cast<uint16_t>(w));
        }
    }
    nb->start[kWords] = static_cast<uint32_t>(nb->words.size());
    g_nb_cache[threshold] = nb;
    return nb;
}

}  // namespace

int build_lookup(const uint8_t *query, int32_t qlen, int32_t threshold, uint32_t *cell_start,
                 uint16_t **offsets, uint32_t *n_offsets) {
    const Neighbourhood *nb = neighbourhood(threshold);
    const int32_t nwords = qlen >= kWordSize ? qlen - kWordSize + 1 : 0;
    std::vector<uint32_t> count(kWords + 1, 0);
    std::vector<int32_t> word_of(static_cast<size_t>(std::max(nwords, 1)));
    for (int32_t i = 0; i < nwords; ++i) {
        const int w = query[i] * 784 + query[i + 1] * 28 + query[i + 2];
        word_of[i] = w;
        for (uint32_t k = nb->start[w]; k < nb->start[w + 1]; ++k) count[nb->words[k]]++;
    }
    uint32_t acc = 0;
    for (int v = 0; v < kWords; ++v) {
        cell_start[v] = acc;
        acc += count[v];
    }
    cell_start[kWords] = acc;
    *n_offsets = acc;
    auto *out = static_cast<uint16_t *>(std::malloc(sizeof(uint16_t) * std::max<uint32_t>(acc, 1)));
    if (!out) return BLAZE_ERR_OUT_OF_MEMORY;
    std::vector<uint32_t> cursor(cell_start, cell_start + kWords);
    // query offsets are visited in increasing order, so every cell ends up sorted
    for (int32_t i = 0; i < nwords; ++i) {
        const int w = word_of[i];
        for (uint32_t k = nb->start[w]; k < nb->start[w + 1]; ++k)
            out[cursor[nb->words[k]]++] = static_cast<uint16_t>(i);
    }
    *offsets = out;
    return BLAZE_OK;
}

void pack_word_cells(const uint32_t *cell_start, uint32_t *pack, uint32_t *presence) {
    std::memset(presence, 0, sizeof(uint32_t) * kPresenceWords);
    for (int w = 0; w < kWords; ++w) {
        const uint32_t cnt = cell_start[w + 1] - cell_start[w];
        pack[w] = (cell_start[w] << 8) | std::min<uint32_t>(cnt, 255u);
        if (cnt) presence[w >> 5] |= 1u << (w & 31);
    }
}

// Karlin-Altschul constants of BLOSUM62 (published NCBI table values).
namespace ka {
constexpr double kUngappedLambda = 0.3176, kUngappedK = 0.134;
constexpr double kGappedLambda = 0.267, kGappedK = 0.041;  // gap open 11, extend 1
constexpr double kGappedAlpha = 1.9, kGappedBeta = -30.0;
constexpr double kLn2 = 0.69314718055994530942;
constexpr double kGapTriggerBits = 22.0;        // blastp default gap trigger
constexpr double kUngappedXdropBits = 7.0;      // blastp default ungapped X-drop
constexpr double kGappedXdropBits = 15.0;       // blastp default preliminary gapped X-drop
}  // namespace ka

// Edge-effect length adjustment: the largest integer ell >= 0 strictly below
// the fixed point of beta + (alpha/lambda)(ln K + ln((m-ell)(n-N ell))) that
// keeps K(m-ell)(n-N ell) above max(m, n) (Altschul & Gish 1996).
static int32_t length_adjustment(double K, double alpha_d_lambda, double beta, int32_t m_len,
                                 uint64_t n_len, uint32_t n_seqs) {
    const double m = m_len, n = static_cast<double>(n_len), N = n_seqs;
    const double logK = std::log(K), floor_sp = std::max(m, n);
    auto feasible = [&](int32_t ell) {
        const double mm = m - ell, nn = n - N * ell;
        if (mm <= 0 || nn <= 0 || K * mm * nn <= floor_sp) return false;
        return beta + alpha_d_lambda * (logK + std::log(mm) + std::log(nn)) > ell;
    };
    int32_t lo = 0, hi = std::max(m_len - 1, 0), best = 0;
    while (lo <= hi) {  // feasible() is true up to the answer and false after it
        const int32_t mid = lo + (hi - lo) / 2;
        if (feasible(mid)) {
            best = mid;
            lo = mid + 1;
        } else {
            hi = mid - 1;
        }
    }
    return best;
}

int default_params(int32_t qlen, uint64_t db_len, uint32_t db_n, double evalue, blaze_params *p) {
    if (!p || qlen <= 0 || evalue <= 0) return BLAZE_ERR_INVALID_ARG;
    using namespace ka;
    std::memset(p, 0, sizeof(*p));
    p->word_threshold = 11;
    p->window = 40;
    p->gap_open = 11;
    p->gap_extend = 1;
    p->ungapped_xdrop = static_cast<int32_t>(std::ceil(kUngappedXdropBits * kLn2 / kUngappedLambda));
    p->gapped_xdrop = static_cast<int32_t>(kGappedXdropBits * kLn2 / kGappedLambda);
    p->lambda = kGappedLambda;
    p->K = kGappedK;
    const int32_t ell = length_adjustment(kGappedK, kGappedAlpha / kGappedLambda, kGappedBeta, qlen,
                                          db_len, db_n);
    const double eff_q = std::max<double>(qlen - ell, 1.0);
    const double eff_db = std::max<double>(static_cast<double>(db_len) - static_cast<double>(db_n) * ell, 1.0);
    p->eff_searchsp = eff_q * eff_db;
    // smallest raw score whose E-value over the search space is <= evalue
    const double s = std::log(kGappedK * p->eff_searchsp / evalue) / kGappedLambda;
    p->gapped_cutoff = std::max<int32_t>(static_cast<int32_t>(std::ceil(s)), 1);
    const int32_t gap_trigger = static_cast<int32_t>(
        (kGapTriggerBits * kLn2 + std::log(kUngappedK)) / kUngappedLambda);
    p->ungapped_cutoff = std::min(gap_trigger, p->gapped_cutoff);
    p->prelim_evalue = evalue;
    p->hitlist_size = 0;
    p->max_hsps = 0;
    return BLAZE_OK;
}

}  // namespace blaze

extern "C" const char *blaze_status_string(int status) {
    switch (status) {
        case BLAZE_OK: return "ok";
        case BLAZE_ERR_INVALID_ARG: return "invalid argument";
        case BLAZE_ERR_CUDA: return "CUDA runtime error";
        case BLAZE_ERR_NO_DEVICE: return "no usable CUDA device";
        case BLAZE_ERR_OUT_OF_MEMORY: return "out of memory";
        case BLAZE_ERR_OUTPUT_TOO_SMALL: return "output buffer too small";
        case BLAZE_ERR_LIMIT: return "request exceeds a library limit";
        case BLAZE_ERR_INTERNAL: return "internal consistency check failed";
        default: return "unknown status";
    }
}

extern "C" int blaze_params_default(int32_t query_length, uint64_t db_residues, uint32_t db_subjects,
                                    double evalue, blaze_params *out) {
    return blaze::default_params(query_length, db_residues, db_subjects, evalue, out);
}
