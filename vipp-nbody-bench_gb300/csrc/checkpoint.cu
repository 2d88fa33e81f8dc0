// Checkpoint files: the state that restarts a run. Host code only (no
// kernels); the layout is documented with gb_checkpoint_info in vipp_gb300.h.
// The reference keeps no checkpoint: its ENABLE_PRINT build writes the
// positions of a run as text (gravity/include/benchmark.hpp:15-20, 46-58).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "checkpoint.h"

namespace gb {
namespace {

constexpr char kMagic[8] = {'V', 'I', 'P', 'P', 'G', 'B', 'C', 'K'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kHeaderBytes = 128;
constexpr uint64_t kMaxParticles = uint64_t(1) << 40;
constexpr uint64_t kMaxSystems = uint64_t(1) << 32;
constexpr size_t kChunkWords = size_t(1) << 20;  // 8 MiB per read or write

// FNV-1a (Fowler, Noll, Vo) over 64-bit little-endian words, one word per round.
struct CheckWord {
    uint64_t h = 0xcbf29ce484222325ull;
    void add(const uint64_t *w, size_t n) {
        for (size_t i = 0; i < n; ++i) h = (h ^ w[i]) * 0x100000001b3ull;
    }
};

bool little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

template <class T>
void put(unsigned char *h, size_t off, T v) {
    std::memcpy(h + off, &v, sizeof(T));
}
template <class T>
T get(const unsigned char *h, size_t off) {
    T v;
    std::memcpy(&v, h + off, sizeof(T));
    return v;
}

// Header layout: 0 magic, 8 version, 12 header bytes, 16 n, 24 nsys, 32 steps,
// 40 t, 48 p, 52 s, 56 precision, 60 mode, 64 flags, 68 leaf parameter in
// effect, 72 eps, 80 G, 88 m, 96..127 zero.
void encode_header(const gb_checkpoint_info &in, unsigned char *h) {
    std::memset(h, 0, kHeaderBytes);
    std::memcpy(h, kMagic, 8);
    put<uint32_t>(h, 8, kVersion);
    put<uint32_t>(h, 12, kHeaderBytes);
    put<uint64_t>(h, 16, in.n);
    put<uint64_t>(h, 24, in.nsys);
    put<int64_t>(h, 32, in.steps);
    put<double>(h, 40, in.t);
    put<int32_t>(h, 48, in.cfg.p);
    put<int32_t>(h, 52, in.cfg.s);
    put<int32_t>(h, 56, in.cfg.precision);
    put<int32_t>(h, 60, in.cfg.mode);
    put<int32_t>(h, 64, in.cfg.flags);
    put<int32_t>(h, 68, in.leaf_s);
    put<double>(h, 72, in.cfg.eps);
    put<double>(h, 80, in.cfg.G);
    put<double>(h, 88, in.cfg.m);
}

int decode_header(const unsigned char *h, gb_checkpoint_info &out, std::string &err) {
    if (std::memcmp(h, kMagic, 8) != 0) return err = "not a checkpoint file (bad magic)", GB_ERR_INVALID;
    if (get<uint32_t>(h, 8) != kVersion)
        return err = "checkpoint version " + std::to_string(get<uint32_t>(h, 8)) + " is not supported", GB_ERR_INVALID;
    if (get<uint32_t>(h, 12) != kHeaderBytes) return err = "checkpoint header size is not 128", GB_ERR_INVALID;
    std::memset(&out, 0, sizeof(out));
    out.n = get<uint64_t>(h, 16);
    out.nsys = get<uint64_t>(h, 24);
    out.steps = get<int64_t>(h, 32);
    out.t = get<double>(h, 40);
    out.cfg.p = get<int32_t>(h, 48);
    out.cfg.s = get<int32_t>(h, 52);
    out.cfg.precision = get<int32_t>(h, 56);
    out.cfg.mode = get<int32_t>(h, 60);
    out.cfg.flags = get<int32_t>(h, 64);
    out.leaf_s = get<int32_t>(h, 68);
    out.cfg.eps = get<double>(h, 72);
    out.cfg.G = get<double>(h, 80);
    out.cfg.m = get<double>(h, 88);
    out.cfg.device = 0;
    if (out.n > kMaxParticles) return err = "checkpoint particle count out of range", GB_ERR_INVALID;
    if (out.nsys == 0 || out.nsys > kMaxSystems) return err = "checkpoint system count out of range", GB_ERR_INVALID;
    if (out.steps < 0) return err = "checkpoint step count is negative", GB_ERR_INVALID;
    return GB_OK;
}

uint64_t body_words(uint64_t n, uint64_t nsys) { return (nsys + 1) + nsys + 6 * n; }

struct File {
    std::FILE *f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

// Writes n 8-byte words from src (copied through a word buffer, so doubles
// are never read as integers in place) and adds them to the check word.
bool write_words(std::FILE *f, const void *src, uint64_t n, CheckWord &cw, std::vector<uint64_t> &buf) {
    const unsigned char *s = static_cast<const unsigned char *>(src);
    while (n) {
        const size_t c = static_cast<size_t>(std::min<uint64_t>(n, kChunkWords));
        buf.resize(c);
        std::memcpy(buf.data(), s, 8 * c);
        cw.add(buf.data(), c);
        if (std::fwrite(buf.data(), 8, c, f) != c) return false;
        n -= c;
        s += 8 * c;
    }
    return true;
}

// Reads n words, adds them to the check word and copies them to dst (when
// not NULL).
bool read_words(std::FILE *f, void *dst, uint64_t n, CheckWord &cw, std::vector<uint64_t> &buf) {
    unsigned char *d = static_cast<unsigned char *>(dst);
    while (n) {
        const size_t c = static_cast<size_t>(std::min<uint64_t>(n, kChunkWords));
        buf.resize(c);
        if (std::fread(buf.data(), 8, c, f) != c) return false;
        cw.add(buf.data(), c);
        if (d) {
            std::memcpy(d, buf.data(), 8 * c);
            d += 8 * c;
        }
        n -= c;
    }
    return true;
}

}  // namespace

int checkpoint_write(const char *path, const gb_checkpoint_info *info, const uint64_t *seg_offsets,
                     const double *m_per_system, const double *x_aos, const double *v_aos, std::string &err) {
    if (!little_endian()) return err = "checkpoints are written on little-endian hosts only", GB_ERR_INVALID;
    if (!path || !*path || !info) return err = "checkpoint needs a path and an info record", GB_ERR_INVALID;
    const uint64_t n = info->n, nsys = info->nsys;
    if (n > kMaxParticles) return err = "particle count out of range", GB_ERR_INVALID;
    if (nsys == 0 || nsys > kMaxSystems) return err = "system count out of range", GB_ERR_INVALID;
    if (info->steps < 0) return err = "step count must be >= 0", GB_ERR_INVALID;
    if (n && (!x_aos || !v_aos)) return err = "null positions or velocities", GB_ERR_INVALID;
    if (!seg_offsets && nsys != 1) return err = "segment offsets are needed for more than one system", GB_ERR_INVALID;
    std::vector<uint64_t> seg(nsys + 1);
    if (seg_offsets) {
        std::memcpy(seg.data(), seg_offsets, sizeof(uint64_t) * (nsys + 1));
    } else {
        seg[0] = 0, seg[1] = n;
    }
    if (seg[0] != 0 || seg[nsys] != n) return err = "segment offsets must run from 0 to n", GB_ERR_INVALID;
    for (uint64_t k = 0; k < nsys; ++k)
        if (seg[k + 1] < seg[k]) return err = "segment offsets must not decrease", GB_ERR_INVALID;
    std::vector<double> m(nsys, info->cfg.m);
    if (m_per_system) std::memcpy(m.data(), m_per_system, sizeof(double) * nsys);

    unsigned char h[kHeaderBytes];
    encode_header(*info, h);
    const std::string tmp = std::string(path) + ".tmp";
    bool ok;
    {
        File out;
        out.f = std::fopen(tmp.c_str(), "wb");
        if (!out.f) return err = "cannot open " + tmp + " for writing", GB_ERR_INVALID;
        CheckWord cw;
        std::vector<uint64_t> buf;
        ok = write_words(out.f, h, kHeaderBytes / 8, cw, buf) && write_words(out.f, seg.data(), nsys + 1, cw, buf) &&
             write_words(out.f, m.data(), nsys, cw, buf) && write_words(out.f, x_aos, 3 * n, cw, buf) &&
             write_words(out.f, v_aos, 3 * n, cw, buf);
        const uint64_t check = cw.h;
        ok = ok && std::fwrite(&check, 8, 1, out.f) == 1 && std::fflush(out.f) == 0;
        ok = std::fclose(out.f) == 0 && ok;
        out.f = nullptr;
    }
    if (!ok) {
        std::remove(tmp.c_str());
        return err = "writing " + tmp + " failed", GB_ERR_INVALID;
    }
    if (std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return err = std::string("cannot rename the checkpoint to ") + path, GB_ERR_INVALID;
    }
    return GB_OK;
}

int checkpoint_read(const char *path, gb_checkpoint_info *info, uint64_t *seg_offsets, double *m_per_system,
                    size_t nsys_cap, double *x_aos, double *v_aos, size_t n_cap, std::string &err) {
    if (!little_endian()) return err = "checkpoints are read on little-endian hosts only", GB_ERR_INVALID;
    if (!path || !info) return err = "checkpoint read needs a path and an info record", GB_ERR_INVALID;
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return err = std::string("cannot open ") + path, GB_ERR_INVALID;
    unsigned char h[kHeaderBytes];
    if (std::fread(h, 1, kHeaderBytes, in.f) != kHeaderBytes) return err = "checkpoint shorter than its header", GB_ERR_INVALID;
    gb_checkpoint_info got;
    int rc = decode_header(h, got, err);
    if (rc) return rc;
    const uint64_t n = got.n, nsys = got.nsys;
    const uint64_t want = kHeaderBytes + 8 * (body_words(n, nsys) + 1);
    if (std::fseek(in.f, 0, SEEK_END) != 0) return err = "cannot seek in the checkpoint", GB_ERR_INVALID;
    const long size = std::ftell(in.f);
    if (size < 0 || static_cast<uint64_t>(size) != want)
        return err = "checkpoint is " + std::to_string(size) + " bytes; its header implies " + std::to_string(want),
               GB_ERR_INVALID;
    *info = got;
    if (!seg_offsets && !m_per_system && !x_aos && !v_aos) return GB_OK;
    if ((seg_offsets || m_per_system) && nsys_cap < nsys)
        return err = "system arrays too small for the checkpoint", GB_ERR_INVALID;
    if ((x_aos || v_aos) && n_cap < n) return err = "particle arrays too small for the checkpoint", GB_ERR_INVALID;
    if (std::fseek(in.f, 0, SEEK_SET) != 0) return err = "cannot seek in the checkpoint", GB_ERR_INVALID;
    CheckWord cw;
    std::vector<uint64_t> buf, seg(nsys + 1);
    bool ok = read_words(in.f, nullptr, kHeaderBytes / 8, cw, buf) && read_words(in.f, seg.data(), nsys + 1, cw, buf) &&
              read_words(in.f, m_per_system, nsys, cw, buf) && read_words(in.f, x_aos, 3 * n, cw, buf) &&
              read_words(in.f, v_aos, 3 * n, cw, buf);
    uint64_t check = 0;
    ok = ok && std::fread(&check, 8, 1, in.f) == 1;
    if (!ok) return err = "checkpoint body could not be read", GB_ERR_INVALID;
    if (check != cw.h) return err = "checkpoint check word does not match its contents (corrupt file)", GB_ERR_INVALID;
    if (seg[0] != 0 || seg[nsys] != n) return err = "checkpoint segment offsets do not run from 0 to n", GB_ERR_INVALID;
    for (uint64_t k = 0; k < nsys; ++k)
        if (seg[k + 1] < seg[k]) return err = "checkpoint segment offsets decrease", GB_ERR_INVALID;
    if (seg_offsets) std::memcpy(seg_offsets, seg.data(), sizeof(uint64_t) * (nsys + 1));
    return GB_OK;
}

}  // namespace gb
