// Checkpoint files (see persist.h).
#include "persist.h"

#include <cstdio>
#include <cstring>
#include <string>

namespace kg {

namespace {

const char kPrpMagic[8] = {'K', 'I', 'T', 'E', 'C', 'K', 'P', '1'};
const char kPrpMagicLegacy[8] = {'A', 'H', 'N', 'C', 'K', 'P', 'T', '1'};
const char kLlrMagic[8] = {'K', 'I', 'T', 'E', 'L', 'L', 'R', '1'};

uint64_t fnv1a(const void *p, size_t len, uint64_t h) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < len; i++) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull;

bool write_atomic(const char *path, const void *hdr, size_t hlen, const std::vector<const std::vector<uint64_t> *> &parts) {
    std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    uint64_t sum = fnv1a(hdr, hlen, kFnvBasis);
    bool ok = std::fwrite(hdr, hlen, 1, f) == 1;
    for (const auto *v : parts) {
        sum = fnv1a(v->data(), v->size() * 8, sum);
        ok = ok && std::fwrite(v->data(), 8, v->size(), f) == v->size();
    }
    ok = ok && std::fwrite(&sum, 8, 1, f) == 1;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path)) {
        std::remove(tmp.c_str());
        return false;
    }
    return true;
}

}  // namespace

bool prp_checkpoint_write(const char *path, uint64_t k, uint64_t n, uint32_t base, uint64_t iter,
                          uint32_t fft_len, const std::vector<uint64_t> &x, const std::vector<uint64_t> &d) {
    PrpCheckpointHeader h;
    std::memcpy(h.magic, kPrpMagic, 8);
    h.k = k;
    h.n = n;
    h.base = base;
    h.iter = iter;
    h.nlimbs = x.size();
    h.fft_len = fft_len;
    return write_atomic(path, &h, sizeof h, {&x, &d});
}

bool prp_checkpoint_header(const char *path, PrpCheckpointHeader &h) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1;
    std::fclose(f);
    return ok && (!std::memcmp(h.magic, kPrpMagic, 8) || !std::memcmp(h.magic, kPrpMagicLegacy, 8));
}

bool prp_checkpoint_read(const char *path, uint64_t k, uint64_t n, uint32_t base, size_t nlimbs,
                         uint64_t &iter, uint32_t &fft_len, std::vector<uint64_t> &x, std::vector<uint64_t> &d) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    PrpCheckpointHeader h;
    std::vector<uint64_t> tx(nlimbs), td(nlimbs);
    uint64_t sum = 0;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 &&
              (!std::memcmp(h.magic, kPrpMagic, 8) || !std::memcmp(h.magic, kPrpMagicLegacy, 8)) &&
              h.k == k && h.n == n && h.base == base && h.nlimbs == nlimbs &&
              std::fread(tx.data(), 8, nlimbs, f) == nlimbs && std::fread(td.data(), 8, nlimbs, f) == nlimbs &&
              std::fread(&sum, 8, 1, f) == 1;
    std::fclose(f);
    if (!ok) return false;
    uint64_t s = fnv1a(&h, sizeof h, kFnvBasis);
    s = fnv1a(tx.data(), nlimbs * 8, s);
    s = fnv1a(td.data(), nlimbs * 8, s);
    if (s != sum) return false;
    iter = h.iter;
    fft_len = (uint32_t)h.fft_len;
    x = tx;
    d = td;
    return true;
}

bool llr_checkpoint_write(const char *path, const LlrCheckpointHeader &h0, const std::vector<uint64_t> &x) {
    LlrCheckpointHeader h = h0;
    std::memcpy(h.magic, kLlrMagic, 8);
    h.nlimbs = x.size();
    return write_atomic(path, &h, sizeof h, {&x});
}

bool llr_checkpoint_read(const char *path, size_t nlimbs, LlrCheckpointHeader &h, std::vector<uint64_t> &x) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::vector<uint64_t> tx(nlimbs);
    uint64_t sum = 0;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && !std::memcmp(h.magic, kLlrMagic, 8) &&
              h.nlimbs == nlimbs && std::fread(tx.data(), 8, nlimbs, f) == nlimbs &&
              std::fread(&sum, 8, 1, f) == 1;
    std::fclose(f);
    if (!ok) return false;
    uint64_t s = fnv1a(&h, sizeof h, kFnvBasis);
    if (fnv1a(tx.data(), nlimbs * 8, s) != sum) return false;
    x = tx;
    return true;
}

bool llr_checkpoint_header(const char *path, LlrCheckpointHeader &h) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    const bool ok = std::fread(&h, sizeof h, 1, f) == 1 && !std::memcmp(h.magic, kLlrMagic, 8);
    std::fclose(f);
    return ok;
}

}  // namespace kg
