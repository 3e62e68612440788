// The PRST proof formats (include/kite_proof.h): giants, fingerprints, state files and the
// positions of the proof points.  These must agree with PRST 14.1 and the reference
// (src/prstproof.c:22-207) byte for byte, so that files written here verify there and the other
// way round; the code is this library's own.
//
// A state file is a sequence of little-endian 32-bit words: the magic 0x9f2b3cd4, the
// application id 4 with the file type in bits 16-23, the fingerprint (omitted when zero), the
// iteration, then per value its word count and its words.  It is written through "<path>.tmp" and
// a rename, and a "<path>.md5" sidecar holds the lowercase hex MD5 of its bytes.
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kite_proof.h"
#include "md5.h"

namespace {

constexpr uint32_t kStateMagic = 0x9f2b3cd4u;
constexpr uint32_t kAppId = 4;

// Little-endian byte buffer of 32-bit words.
class Words {
  public:
    void word(uint32_t v) {
        for (int s = 0; s < 32; s += 8) bytes_.push_back((uint8_t)(v >> s));
    }
    void giant(const pp_giant &g) {
        word((uint32_t)g.len);
        for (int32_t i = 0; i < g.len; i++) word(g.w[i]);
    }
    const std::vector<uint8_t> &bytes() const { return bytes_; }

  private:
    std::vector<uint8_t> bytes_;
};

// Reader over a file's bytes; every get fails once the bytes run out.
class Cursor {
  public:
    explicit Cursor(const std::vector<uint8_t> &b) : b_(b) {}
    bool word(uint32_t &v) {
        if (at_ + 4 > b_.size()) return false;
        v = (uint32_t)b_[at_] | (uint32_t)b_[at_ + 1] << 8 | (uint32_t)b_[at_ + 2] << 16 | (uint32_t)b_[at_ + 3] << 24;
        at_ += 4;
        return true;
    }
    bool done() const { return at_ == b_.size(); }
    size_t left() const { return b_.size() - at_; }

  private:
    const std::vector<uint8_t> &b_;
    size_t at_ = 0;
};

bool put_file(const std::string &path, const void *data, size_t len) {
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(data, 1, len, f) == len && std::fflush(f) == 0 && fsync(fileno(f)) == 0;
    ok = std::fclose(f) == 0 && ok;
    if (ok && std::rename(tmp.c_str(), path.c_str()) == 0) return true;
    std::remove(tmp.c_str());
    return false;
}

bool get_file(const std::string &path, std::vector<uint8_t> &out) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    uint8_t chunk[1 << 16];
    for (size_t got; (got = std::fread(chunk, 1, sizeof chunk, f)) > 0;) out.insert(out.end(), chunk, chunk + got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

uint32_t md5_word0(kg::Md5 &m) {
    uint8_t d[16];
    m.digest(d);
    return (uint32_t)d[0] | (uint32_t)d[1] << 8 | (uint32_t)d[2] << 16 | (uint32_t)d[3] << 24;
}

}  // namespace

extern "C" {

void pp_giant_free(pp_giant *g) {
    if (!g) return;
    std::free(g->w);
    *g = pp_giant{nullptr, 0};
}

uint64_t pp_res64(const pp_giant *g) {
    uint64_t r = 0;
    for (int32_t i = 0; i < 2 && i < g->len; i++) r |= (uint64_t)g->w[i] << (32 * i);
    return r;
}

// N mod 3417905339 for N = k*2^n - 1
uint32_t pp_fingerprint(uint64_t k, uint64_t n) {
    const uint64_t p = 3417905339u;
    uint64_t pow2 = 1, sq = 2;
    for (uint64_t e = n; e; e >>= 1, sq = sq * sq % p)
        if (e & 1) pow2 = pow2 * sq % p;
    return (uint32_t)((k % p * pow2 + p - 1) % p);
}

uint32_t pp_unique_fingerprint(uint32_t fp, const char *id) {
    const uint8_t f[4] = {(uint8_t)fp, (uint8_t)(fp >> 8), (uint8_t)(fp >> 16), (uint8_t)(fp >> 24)};
    kg::Md5 m;
    m.update(f, 4);
    m.update(id, std::strlen(id));
    return md5_word0(m);
}

uint32_t pp_proof_fingerprint(uint64_t k, uint64_t n, uint32_t a) {
    const std::string id = std::to_string(a) + "." + std::to_string(n);
    return pp_unique_fingerprint(pp_fingerprint(k, n), id.c_str());
}

int pp_write(const char *path, int type, uint32_t fingerprint, int32_t iteration, const pp_giant *g, int ng) {
    Words w;
    w.word(kStateMagic);
    w.word(kAppId | (uint32_t)(uint8_t)type << 16);
    if (fingerprint) w.word(fingerprint);
    w.word((uint32_t)iteration);
    for (int i = 0; i < ng; i++) w.giant(g[i]);
    const std::vector<uint8_t> &b = w.bytes();
    const std::string hex = kg::Md5::hex(b.data(), b.size());
    const std::string p(path);
    return put_file(p, b.data(), b.size()) && put_file(p + ".md5", hex.data(), hex.size()) ? 0 : -1;
}

int pp_read(const char *path, int type, uint32_t fingerprint, int32_t *iteration, pp_giant *g, int maxg) {
    for (int i = 0; i < maxg; i++) g[i] = pp_giant{nullptr, 0};
    std::vector<uint8_t> b, sidecar;
    if (!get_file(path, b)) return -1;
    // a sidecar that is present must hold the file's MD5
    if (get_file(std::string(path) + ".md5", sidecar)) {
        const std::string hex = kg::Md5::hex(b.data(), b.size());
        if (sidecar.size() < 32 || std::memcmp(hex.data(), sidecar.data(), 32) != 0) return -1;
    }
    Cursor c(b);
    uint32_t v = 0;
    if (!c.word(v) || v != kStateMagic) return -1;
    if (!c.word(v) || (v & 0xff) != kAppId || ((v >> 16) & 0xff) != (uint32_t)type) return -1;
    if (fingerprint && (!c.word(v) || v != fingerprint)) return -1;
    if (!c.word(v)) return -1;
    *iteration = (int32_t)v;
    for (int i = 0; i < maxg && !c.done(); i++) {  // trailing values may be absent
        uint32_t len = 0;
        if (!c.word(len) || (int32_t)len < 0 || (size_t)len * 4 > c.left()) {
            for (int j = 0; j < maxg; j++) pp_giant_free(&g[j]);
            return -1;
        }
        g[i].w = static_cast<uint32_t *>(std::malloc(4 * (size_t)len + 4));
        g[i].len = (int32_t)len;
        for (uint32_t j = 0; j < len; j++) c.word(g[i].w[j]);
    }
    return 0;
}

// Point i of count = 2^t points (0 < i < count) along T iterations: with i's bits b_1..b_t read
// from the top and S the position of its lowest set bit, pos[i] = sum over s = 1..S of
// b_s * floor(T / 2^s) + bit s-1 of T.  This is PRST's recursive halving of the span, where
// every halving of an odd span rounds up.  The return value is the last span, floor(T / 2^t).
int pp_points(uint32_t iterations, int count, uint32_t *pos) {
    int t = 0;
    while ((1 << t) < count) t++;
    pos[0] = 0;
    for (int i = 1; i < count; i++) {
        const int S = t - __builtin_ctz((unsigned)i);
        uint32_t p = 0;
        for (int s = 1; s <= S; s++) {
            if ((i >> (t - s)) & 1) p += iterations >> s;
            p += (iterations >> (s - 1)) & 1;
        }
        pos[i] = p;
    }
    pos[count] = iterations;
    return count > 1 ? (int)(iterations >> t) : 0;
}

}  // extern "C"
