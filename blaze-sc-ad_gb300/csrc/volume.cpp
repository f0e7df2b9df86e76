// volume.cpp -- reader of NCBI BLAST protein database volumes (.pin index +
// .psq sequence file) into the resident device database, in place of the
// per-subject BlastSeqSrcGetSequence gathers of the reference
// (BLAZE_gpu/gpuBLAZE.cu:1587-1611, which copies every subject into a pinned
// staging buffer for every chunk of every search).
//
// Layout read (NCBI BLAST database format, protein volume; integers in the
// index are big-endian except the 8-byte total length, which is
// little-endian):
//   .pin  version (4 or 5), database type (1 = protein),
//         [version 5: volume number], title (length-prefixed string),
//         [version 5: LMDB file name (string)], creation date (string),
//         number of sequences N, total residues (8 bytes), longest sequence,
//         N+1 header offsets into .phr, N+1 sequence offsets into .psq
//   .psq  NCBIstdaa residues; sequence i occupies [off[i], off[i+1] - 1),
//         each followed by one 0 byte (the file also starts with one)
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "blaze_prelim.h"
#include "internal.h"

namespace {

struct Volume {
    uint32_t version = 0, n = 0, max_len = 0;
    uint64_t total = 0;
    std::vector<uint32_t> seq_off;  // N + 1
};

bool read_file(const std::string &path, std::vector<uint8_t> &out) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

struct Cursor {
    const std::vector<uint8_t> &b;
    size_t pos = 0;
    bool ok = true;
    uint32_t be32() {
        if (pos + 4 > b.size()) {
            ok = false;
            return 0;
        }
        const uint32_t v = (uint32_t{b[pos]} << 24) | (uint32_t{b[pos + 1]} << 16) | (uint32_t{b[pos + 2]} << 8) |
                           uint32_t{b[pos + 3]};
        pos += 4;
        return v;
    }
    uint64_t le64() {
        if (pos + 8 > b.size()) {
            ok = false;
            return 0;
        }
        uint64_t v = 0;
        for (int i = 7; i >= 0; --i) v = (v << 8) | b[pos + i];
        pos += 8;
        return v;
    }
    void skip_string() {
        const uint32_t len = be32();
        if (!ok || pos + len > b.size()) {
            ok = false;
            return;
        }
        pos += len;
    }
};

int parse_index(const std::string &base, Volume &v) {
    std::vector<uint8_t> pin;
    if (!read_file(base + ".pin", pin)) return BLAZE_ERR_INVALID_ARG;
    Cursor c{pin};
    v.version = c.be32();
    if (!c.ok || (v.version != 4 && v.version != 5)) return BLAZE_ERR_INVALID_ARG;
    if (c.be32() != 1) return BLAZE_ERR_INVALID_ARG;  // not a protein database
    if (v.version == 5) c.be32();                     // volume number
    c.skip_string();                                  // title
    if (v.version == 5) c.skip_string();              // LMDB file name
    c.skip_string();                                  // date
    v.n = c.be32();
    v.total = c.le64();
    v.max_len = c.be32();
    if (!c.ok) return BLAZE_ERR_INVALID_ARG;
    const size_t need = 2 * (static_cast<size_t>(v.n) + 1) * 4;
    if (c.pos + need > pin.size()) return BLAZE_ERR_INVALID_ARG;
    c.pos += (static_cast<size_t>(v.n) + 1) * 4;  // header offsets (.phr): not needed here
    v.seq_off.resize(static_cast<size_t>(v.n) + 1);
    for (auto &o : v.seq_off) o = c.be32();
    uint64_t total = 0;
    for (uint32_t i = 0; i < v.n; ++i) {
        if (v.seq_off[i + 1] <= v.seq_off[i]) return BLAZE_ERR_INVALID_ARG;  // each holds its 0 separator
        total += v.seq_off[i + 1] - v.seq_off[i] - 1;
    }
    if (total != v.total) return BLAZE_ERR_INVALID_ARG;  // the header disagrees with the offsets
    return BLAZE_OK;
}

// Size of a file in bytes, or -1.
long long file_size(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return -1;
    long long n = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) n = static_cast<long long>(std::ftell(f));
    std::fclose(f);
    return n;
}

}  // namespace

extern "C" int blaze_volume_info(const char *path, uint32_t *n_subjects, uint64_t *total_residues,
                                 uint32_t *max_length) try {
    if (!path) return BLAZE_ERR_INVALID_ARG;
    Volume v;
    const int rc = parse_index(path, v);
    if (rc != BLAZE_OK) return rc;
    if (n_subjects) *n_subjects = v.n;
    if (total_residues) *total_residues = v.total;
    if (max_length) *max_length = v.max_len;
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_volume_read(const char *path, uint8_t *residues, uint64_t capacity, uint64_t *offsets) try {
    if (!path || !offsets) return BLAZE_ERR_INVALID_ARG;
    Volume v;
    int rc = parse_index(path, v);
    if (rc != BLAZE_OK) return rc;
    std::vector<uint8_t> psq;
    if (!read_file(std::string(path) + ".psq", psq)) return BLAZE_ERR_INVALID_ARG;
    if (v.n && v.seq_off[v.n] > psq.size()) return BLAZE_ERR_INVALID_ARG;  // shorter than the index says
    const uint64_t total = v.total;
    if (capacity < total) return BLAZE_ERR_OUTPUT_TOO_SMALL;
    if (total && !residues) return BLAZE_ERR_INVALID_ARG;
    uint64_t at = 0;
    offsets[0] = 0;
    for (uint32_t i = 0; i < v.n; ++i) {
        const uint32_t len = v.seq_off[i + 1] - v.seq_off[i] - 1;
        std::memcpy(residues + at, psq.data() + v.seq_off[i], len);
        at += len;
        offsets[i + 1] = at;
    }
    return BLAZE_OK;
} BLAZE_ABI_CATCH

extern "C" int blaze_db_open(int device, const char *path, blaze_db **out) try {
    if (!out) return BLAZE_ERR_INVALID_ARG;
    *out = nullptr;
    uint32_t n = 0, max_len = 0;
    uint64_t total = 0;
    int rc = blaze_volume_info(path, &n, &total, &max_len);
    if (rc != BLAZE_OK) return rc;
    // the host copies below are sized by the index: the sequence file must
    // hold what it claims (a residue and a separator per subject, at least)
    const long long psq_bytes = file_size(std::string(path) + ".psq");
    if (psq_bytes < 0 || total + n > static_cast<unsigned long long>(psq_bytes)) return BLAZE_ERR_INVALID_ARG;
    std::vector<uint8_t> res(std::max<uint64_t>(total, 1));
    std::vector<uint64_t> off(static_cast<size_t>(n) + 1);
    rc = blaze_volume_read(path, res.data(), total, off.data());
    if (rc != BLAZE_OK) return rc;
    return blaze_db_create(device, res.data(), off.data(), n, out);
} BLAZE_ABI_CATCH
