// PRST-compatible Fermat proofs (include/kite_proof.h) on the GB300 engine.
//
// The proof is Pietrzak's verifiable-delay-function proof in the form PRST 14.1 uses for
// k*2^n-1 (its src/proof.cpp; the reference restates it in src/prstproof.c).  A Fermat test
// x_{i+1} = x_i^2 from x_0 = a^k leaves count+1 points x_{pos[i]}; the save step folds them
// level by level into t = log2(count) products, each level's challenge being MD5 over the
// running value Y and the new product; the build step applies the same challenges to x_0 and Y
// and writes the certificate X with Y = X^(2^M); the verify step recomputes X^(2^M).
//
// Every number operation is a kite_* call on the caller's context, so products, exponentiations
// and the certificate squarings run on the GPU; file I/O, MD5 and the challenges are host work.
// The file bytes, names, challenges and error texts match the reference's, so the files it
// writes are interchangeable with the reference's and PRST's.
#include "../../include/kite_proof.h"

#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kite_internal.h"
#include "md5.h"

namespace {

constexpr uint32_t kMagic = 0x9f2b3cd4u;  // PRST TaskState magic
constexpr uint32_t kAppId = 4;
constexpr double kRoundoffLimit = 0.40;

using u128 = unsigned __int128;

// A kite number freed with its scope.
struct Num {
    kite_ctx *ctx;
    kite_num *x;
    explicit Num(kite_ctx *c) : ctx(c), x(kite_num_new(c)) {}
    ~Num() {
        if (x) kite_num_free(ctx, x);
    }
    Num(const Num &) = delete;
    Num &operator=(const Num &) = delete;
    operator kite_num *() const { return x; }
};

// A giant owned by its scope.
struct Giant {
    pp_giant g{nullptr, 0};
    ~Giant() { pp_giant_free(&g); }
    Giant() = default;
    Giant(const Giant &) = delete;
    Giant &operator=(const Giant &) = delete;
};

void put32(std::vector<uint8_t> &b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i)));
}

uint32_t get32(const uint8_t *p) {
    return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

// The words of a giant as little-endian bytes (the on-disk and hashed form).
std::vector<uint8_t> giant_bytes(const pp_giant &g) {
    std::vector<uint8_t> b;
    b.reserve(4 * (size_t)std::max(g.len, 0));
    for (int32_t i = 0; i < g.len; i++) put32(b, g.w[i]);
    return b;
}

// Write through "<path>.tmp", flushed to disk, then renamed over the target.
bool write_atomic(const std::string &path, const void *p, size_t n) {
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(p, 1, n, f) == n;
    ok = ok && std::fflush(f) == 0 && fsync(fileno(f)) == 0;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        return false;
    }
    return true;
}

bool read_all(const std::string &path, std::vector<uint8_t> &out) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

void remove_with_md5(const std::string &path) {
    std::remove(path.c_str());
    std::remove((path + ".md5").c_str());
}

std::string point_path(const char *prefix, const char *kind, int index) {
    return std::string(prefix) + "." + kind + "." + std::to_string(index);
}

// Reads <prefix>.<kind>.<index>, which must carry iteration `expect`; prints the reference's
// message otherwise.
bool read_value(const char *prefix, const char *kind, int index, int type, uint32_t fp, int32_t expect,
                pp_giant *g) {
    const std::string path = point_path(prefix, kind, index);
    int32_t it = 0;
    if (pp_read(path.c_str(), type, fp, &it, g, 1) != 0 || it != expect) {
        if (g->w) pp_giant_free(g);
        std::fprintf(stderr, "%s is missing or corrupt.\n", path.c_str());
        return false;
    }
    return true;
}

int depth_of(int count) {
    int t = 0;
    while ((1 << t) < count) t++;
    return t;
}

bool is_small_prime(unsigned p) {
    if (p < 2) return false;
    for (unsigned q = 2; q * q <= p; q++)
        if (p % q == 0) return false;
    return true;
}

// The challenge of one level: the first 64 bits of MD5(fp || Y || D) as two little-endian
// words, the low word made odd and the high word non-zero, then stepped by 2 until no prime
// below 1000 divides it (PRST proof.cpp hash_giants and make_prime; src/prstproof.c:247-278).
u128 challenge(uint32_t fp, const pp_giant &Y, const pp_giant &D) {
    kg::Md5 m;
    uint8_t f[4];
    for (int i = 0; i < 4; i++) f[i] = (uint8_t)(fp >> (8 * i));
    m.update(f, 4);
    const std::vector<uint8_t> yb = giant_bytes(Y), db = giant_bytes(D);
    if (!yb.empty()) m.update(yb.data(), yb.size());
    if (!db.empty()) m.update(db.data(), db.size());
    uint8_t d[16];
    m.digest(d);
    uint32_t lo = get32(d) | 1u, hi = get32(d + 4);
    if (hi == 0) hi = 1;
    u128 g = (u128)hi << 32 | lo;
    static const std::vector<unsigned> primes = [] {
        std::vector<unsigned> v;
        for (unsigned p = 2; p < 1000; p++)
            if (is_small_prime(p)) v.push_back(p);
        return v;
    }();
    for (;;) {
        bool hit = false;
        for (unsigned p : primes)
            if (g % p == 0) {
                hit = true;
                break;
            }
        if (!hit) return g;
        g += 2;
    }
}

// X = X0^e by left-to-right binary powering; X and X0 are distinct numbers.
void power(kite_ctx *ctx, u128 e, kite_num *X, const kite_num *X0) {
    int top = 0;
    while (top < 128 && (e >> top) > 1) top++;
    kite_copy(ctx, X, X0);
    for (int bit = top - 1; bit >= 0; bit--) {
        kite_square(ctx, X);
        if ((e >> bit) & 1) kite_mul(ctx, X, X0);
    }
}

bool roundoff_ok(kite_ctx *ctx) { return kite_max_roundoff(ctx) < kRoundoffLimit; }

bool giants_equal(const pp_giant &a, const pp_giant &b) {
    return a.len == b.len && (a.len == 0 || std::memcmp(a.w, b.w, 4 * (size_t)a.len) == 0);
}

bool is_one(const std::vector<uint64_t> &l) {
    if (l.empty() || l[0] != 1) return false;
    for (size_t i = 1; i < l.size(); i++)
        if (l[i]) return false;
    return true;
}

uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

// (N - 1) mod m = (k*2^n - 2) mod m
uint64_t nm1_mod(uint64_t k, uint64_t n, uint64_t m) {
    uint64_t r = 1 % m, b = 2 % m;
    for (uint64_t e = n; e; e >>= 1, b = mulmod64(b, b, m))
        if (e & 1) r = mulmod64(r, b, m);
    return (mulmod64(k % m, r, m) + 2 * m - 2 % m) % m;
}

// PRST's check for a composite result (proof.cpp:82, security 24): R = a^(N-1) must not be a
// root of unity of the small order made of 2 (the power of 2 in N-1 is 2^1) and, for every odd
// prime p < 2^12 dividing N-1, the largest p^e dividing N-1 below 2^31.  `xn` is the last point
// a^(N+1).  A probable prime passes unchecked.  true when the check passes.
bool roots_of_unity_ok(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, const pp_giant &xn) {
    const size_t nl = ctx->lay.nlimbs;
    std::vector<uint64_t> l(nl, 0);
    for (int32_t i = 0; i < xn.len && (size_t)i < 2 * nl; i++) l[i / 2] |= (uint64_t)xn.w[i] << (32 * (i & 1));
    if (kg::residue_nm1(l.data(), ctx->lay.Nl.data(), nl, a) != 0) return true;
    if (is_one(l)) return true;
    Num R(ctx), X(ctx), T(ctx);
    kite_set_limbs(ctx, R, l.data());
    kite_copy(ctx, X, R);
    kite_square(ctx, X);
    for (uint32_t p = 3; p < 4096; p += 2) {
        if (!is_small_prime(p) || nm1_mod(k, n, p) != 0) continue;
        uint64_t d = p;
        while (d * p < 2147483647u && nm1_mod(k, n, d * p) == 0) d *= p;
        kite_copy(ctx, T, X);  // X = X^d
        int top = 0;
        while ((d >> top) > 1) top++;
        for (int b = top - 1; b >= 0; b--) {
            kite_square(ctx, X);
            if ((d >> b) & 1) kite_mul(ctx, X, T);
        }
    }
    kite_get_limbs(ctx, X, l.data());
    return !is_one(l);
}

}  // namespace

extern "C" {

void pp_giant_free(pp_giant *g) {
    if (!g) return;
    std::free(g->w);
    g->w = nullptr;
    g->len = 0;
}

uint32_t pp_fingerprint(uint64_t k, uint64_t n) {
    const uint64_t p = 3417905339u;
    uint64_t r = 1, b = 2;
    for (uint64_t e = n; e; e >>= 1, b = b * b % p)
        if (e & 1) r = r * b % p;
    return (uint32_t)(((k % p) * r % p + p - 1) % p);
}

uint32_t pp_unique_fingerprint(uint32_t fp, const char *id) {
    kg::Md5 m;
    uint8_t f[4];
    for (int i = 0; i < 4; i++) f[i] = (uint8_t)(fp >> (8 * i));
    m.update(f, 4);
    m.update(id, std::strlen(id));
    uint8_t d[16];
    m.digest(d);
    return get32(d);
}

uint32_t pp_proof_fingerprint(uint64_t k, uint64_t n, uint32_t a) {
    const std::string id = std::to_string(a) + "." + std::to_string(n);
    return pp_unique_fingerprint(pp_fingerprint(k, n), id.c_str());
}

int pp_write(const char *path, int type, uint32_t fingerprint, int32_t iteration, const pp_giant *g, int ng) {
    std::vector<uint8_t> b;
    put32(b, kMagic);
    put32(b, kAppId | (uint32_t)(uint8_t)type << 16);
    if (fingerprint) put32(b, fingerprint);
    put32(b, (uint32_t)iteration);
    for (int i = 0; i < ng; i++) {
        put32(b, (uint32_t)g[i].len);
        const std::vector<uint8_t> w = giant_bytes(g[i]);
        b.insert(b.end(), w.begin(), w.end());
    }
    const std::string hex = kg::Md5::hex(b.data(), b.size());
    const std::string p(path);
    if (!write_atomic(p, b.data(), b.size())) return -1;
    return write_atomic(p + ".md5", hex.data(), hex.size()) ? 0 : -1;
}

int pp_read(const char *path, int type, uint32_t fingerprint, int32_t *iteration, pp_giant *g, int maxg) {
    for (int i = 0; i < maxg; i++) g[i] = pp_giant{nullptr, 0};
    std::vector<uint8_t> b, m;
    if (!read_all(path, b)) return -1;
    if (read_all(std::string(path) + ".md5", m)) {  // a sidecar that is present must match
        const std::string hex = kg::Md5::hex(b.data(), b.size());
        if (m.size() < 32 || std::memcmp(hex.data(), m.data(), 32) != 0) return -1;
    }
    size_t off = 0;
    auto get = [&](uint32_t &v) {
        if (off + 4 > b.size()) return false;
        v = get32(b.data() + off);
        off += 4;
        return true;
    };
    uint32_t v;
    if (!get(v) || v != kMagic) return -1;
    if (!get(v) || (v & 0xff) != kAppId || ((v >> 16) & 0xff) != (uint32_t)type) return -1;
    if (fingerprint && (!get(v) || v != fingerprint)) return -1;
    if (!get(v)) return -1;
    *iteration = (int32_t)v;
    for (int i = 0; i < maxg; i++) {
        if (off == b.size()) continue;  // optional trailing values (certificate a_power, a_base)
        uint32_t len;
        if (!get(len) || (int32_t)len < 0 || off + 4 * (size_t)len > b.size()) {
            for (int j = 0; j <= i; j++) pp_giant_free(&g[j]);
            return -1;
        }
        g[i].w = static_cast<uint32_t *>(std::malloc(4 * (size_t)len + 4));
        g[i].len = (int32_t)len;
        for (uint32_t j = 0; j < len; j++) g[i].w[j] = get32(b.data() + off + 4 * (size_t)j);
        off += 4 * (size_t)len;
    }
    return 0;
}

int pp_points(uint32_t iterations, int count, uint32_t *pos) {
    // Point i sits at the binary-subdivision position of i/count along the iterations; every
    // halving of an odd span rounds its first half up (PRST proof.cpp:160).
    int M = 0;
    pos[0] = 0;
    for (int i = 1; i < count; i++) {
        M = (int)iterations;
        pos[i] = 0;
        for (int half = count / 2; half > 0 && (i & (half * 2 - 1)) != 0; half >>= 1) {
            M /= 2;
            if (i & half) pos[i] += (uint32_t)M;
            if (iterations & (uint32_t)(count / half / 2)) pos[i]++;
        }
    }
    pos[count] = iterations;
    return M;
}

void pp_from_num(kite_ctx *ctx, const kite_num *x, pp_giant *g) {
    const size_t nl = kite_limbs(ctx);
    std::vector<uint64_t> l(nl);
    kite_get_limbs(ctx, x, l.data());
    g->w = static_cast<uint32_t *>(std::malloc(nl * 8 + 4));
    for (size_t i = 0; i < nl; i++) {
        g->w[2 * i] = (uint32_t)l[i];
        g->w[2 * i + 1] = (uint32_t)(l[i] >> 32);
    }
    g->len = (int32_t)(2 * nl);
    while (g->len > 0 && g->w[g->len - 1] == 0) g->len--;
}

void pp_to_num(kite_ctx *ctx, const pp_giant *g, kite_num *x) {
    const size_t nl = kite_limbs(ctx);
    std::vector<uint64_t> l(nl, 0);
    for (int32_t i = 0; i < g->len && (size_t)i < 2 * nl; i++) l[i / 2] |= (uint64_t)g->w[i] << (32 * (i & 1));
    kite_set_limbs(ctx, x, l.data());
}

uint64_t pp_res64(const pp_giant *g) {
    uint64_t r = 0;
    if (g->len > 0) r = g->w[0];
    if (g->len > 1) r |= (uint64_t)g->w[1] << 32;
    return r;
}

int pp_save_products(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count, const char *prefix, int keep,
                     volatile int *abort_flag, uint64_t *raw_res64) {
    const uint32_t fpN = pp_fingerprint(k, n), fpP = pp_proof_fingerprint(k, n, a);
    const int t = depth_of(count);
    std::vector<uint32_t> pos(count + 1);
    pp_points((uint32_t)n, count, pos.data());
    Num Y(ctx), D(ctx), T(ctx);
    std::vector<Num *> tree;
    for (int i = 0; i < t; i++) tree.push_back(new Num(ctx));
    struct Free {
        std::vector<Num *> &v;
        ~Free() {
            for (Num *p : v) delete p;
        }
    } free_tree{tree};
    std::vector<u128> h(t, 0);
    kite_reset_roundoff(ctx);
    auto aborted = [&] { return abort_flag && *abort_flag; };
    {
        Giant g;
        if (!read_value(prefix, "proof", count, PP_TYPE_VALUE, fpP, (int32_t)pos[count], &g.g)) return -1;
        pp_to_num(ctx, &g.g, Y);
    }
    // Y folds in one product per level: Y <- Y * D_i^h_i, h_i = challenge(Y, D_i).
    auto fold = [&](int level, const pp_giant &dg) {
        Giant yg;
        pp_from_num(ctx, Y, &yg.g);
        h[level] = challenge(fpN, yg.g, dg);
        power(ctx, h[level], T, D);
        kite_mul(ctx, Y, T);
    };
    // products left by an interrupted run: each finished level costs one power, not a redo
    int first = 0;
    for (; first < t; first++) {
        Giant dg;
        int32_t it = 0;
        const std::string path = point_path(prefix, "prod", first);
        if (pp_read(path.c_str(), PP_TYPE_PRODUCT, fpP, &it, &dg.g, 1) != 0 || it != first) break;
        pp_to_num(ctx, &dg.g, D);
        fold(first, dg.g);
    }
    for (int i = first; i < t; i++) {
        if (aborted()) return PP_ABORTED;
        if (i == 0) {
            Giant g;
            if (!read_value(prefix, "proof", count / 2, PP_TYPE_VALUE, fpP, (int32_t)pos[count / 2], &g.g)) return -1;
            pp_to_num(ctx, &g.g, D);
        } else {
            // level i combines the 2^i points at odd multiples of count / 2^(i+1); tree[l] keeps
            // the partial product of an unfinished subtree at depth l, raised by h[l] when its
            // sibling completes
            for (int j = 0; j < (1 << i); j++) {
                if (aborted()) return PP_ABORTED;
                const int idx = (1 + 2 * j) << (t - i - 1);
                Giant g;
                if (!read_value(prefix, "proof", idx, PP_TYPE_VALUE, fpP, (int32_t)pos[idx], &g.g)) return -1;
                pp_to_num(ctx, &g.g, D);
                for (int up = 1; up <= i; up++) {
                    if (!((j >> (up - 1)) & 1)) {
                        kite_copy(ctx, *tree[i - up], D);
                        break;
                    }
                    power(ctx, h[i - up], T, *tree[i - up]);
                    kite_mul(ctx, D, T);
                }
            }
        }
        Giant dg;
        pp_from_num(ctx, D, &dg.g);
        const std::string path = point_path(prefix, "prod", i);
        if (pp_write(path.c_str(), PP_TYPE_PRODUCT, fpP, i, &dg.g, 1)) {
            std::fprintf(stderr, "Write to %s failed.\n", path.c_str());
            return -1;
        }
        fold(i, dg.g);
        if (!roundoff_ok(ctx)) {
            std::fprintf(stderr, "round-off error while compressing proof points.\n");
            return -1;
        }
    }
    {
        Giant yg;
        pp_from_num(ctx, Y, &yg.g);
        *raw_res64 = pp_res64(&yg.g);
    }
    if (!keep)
        for (int i = 1; i < count; i++) remove_with_md5(point_path(prefix, "proof", i));
    return 0;
}

int pp_build_cert(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count, const char *prefix, int keep,
                  uint64_t *cert_res64) {
    const uint32_t fpN = pp_fingerprint(k, n), fpP = pp_proof_fingerprint(k, n, a);
    const int t = depth_of(count);
    std::vector<uint32_t> pos(count + 1);
    pp_points((uint32_t)n, count, pos.data());
    Num X(ctx), Y(ctx), D(ctx), T(ctx);
    kite_reset_roundoff(ctx);
    {
        // point 0 must be a^k
        Giant g, dg;
        if (!read_value(prefix, "proof", 0, PP_TYPE_VALUE, fpP, 0, &g.g)) return -1;
        pp_to_num(ctx, &g.g, X);
        kite_set_u64(ctx, T, a);
        kite_set_u64(ctx, D, 1);
        for (int b = 63; b >= 0; b--) {
            kite_square(ctx, D);
            if ((k >> b) & 1) kite_mul(ctx, D, T);
        }
        pp_from_num(ctx, D, &dg.g);
        if (!giants_equal(g.g, dg.g)) {
            std::fprintf(stderr, "invalid a^k.\n");
            return -1;
        }
    }
    {
        Giant g;
        if (!read_value(prefix, "proof", count, PP_TYPE_VALUE, fpP, (int32_t)pos[count], &g.g)) return -1;
        pp_to_num(ctx, &g.g, Y);
        if (!roots_of_unity_ok(ctx, k, n, a, g.g)) {
            std::fprintf(stderr, "roots of unity check failed.\n");
            return -1;
        }
    }
    // level i: X <- X^(h_i * b) * D_i with b = 2 when the span M is odd, Y <- Y * D_i^h_i
    uint32_t M = pos[count];
    for (int i = 0; i < t; i++, M >>= 1) {
        Giant dg, yg;
        if (!read_value(prefix, "prod", i, PP_TYPE_PRODUCT, fpP, i, &dg.g)) return -1;
        pp_to_num(ctx, &dg.g, D);
        pp_from_num(ctx, Y, &yg.g);
        const u128 h = challenge(fpN, yg.g, dg.g);
        power(ctx, h * (M % 2 ? 2 : 1), T, X);
        kite_copy(ctx, X, T);
        kite_mul(ctx, X, D);
        power(ctx, h, T, D);
        kite_mul(ctx, Y, T);
        if (!roundoff_ok(ctx)) {
            std::fprintf(stderr, "round-off error while building the certificate.\n");
            return -1;
        }
    }
    {
        Giant yg;
        pp_from_num(ctx, Y, &yg.g);
        if (yg.g.len == 0) {
            std::fprintf(stderr, "invalid proof, the certificate is zero.\n");
            return -1;
        }
        *cert_res64 = pp_res64(&yg.g);
    }
    {
        // the certificate: X, then the empty a_power and a_base of a smooth test
        pp_giant c[3] = {{nullptr, 0}, {nullptr, 0}, {nullptr, 0}};
        pp_from_num(ctx, X, &c[0]);
        const std::string path = std::string(prefix) + ".cert";
        const int w = pp_write(path.c_str(), PP_TYPE_CERT, fpN, (int32_t)M, c, 3);
        pp_giant_free(&c[0]);
        if (w) {
            std::fprintf(stderr, "Write to %s failed.\n", path.c_str());
            return -1;
        }
    }
    if (!keep) {
        remove_with_md5(point_path(prefix, "proof", 0));
        remove_with_md5(point_path(prefix, "proof", count));
        for (int i = 0; i < t; i++) remove_with_md5(point_path(prefix, "prod", i));
    }
    return 0;
}

int pp_verify_cert(kite_ctx *ctx, uint64_t k, uint64_t n, const char *path, uint64_t *cert_res64, uint32_t *Mout) {
    pp_giant c[3];
    int32_t M = 0;
    if (pp_read(path, PP_TYPE_CERT, pp_fingerprint(k, n), &M, c, 3) != 0 || M < 0) {
        if (M < 0)
            for (auto &g : c) pp_giant_free(&g);
        std::fprintf(stderr, "Invalid certificate file.\n");
        return -1;
    }
    const bool li = c[1].len != 0;
    pp_giant_free(&c[1]);
    pp_giant_free(&c[2]);
    if (li) {  // Gerbicz-Li certificates come from non-smooth tests
        pp_giant_free(&c[0]);
        std::fprintf(stderr, "Gerbicz-Li certificates are not supported.\n");
        return -1;
    }
    Num x0(ctx), x(ctx), d(ctx), e(ctx);
    pp_to_num(ctx, &c[0], x0);
    pp_giant_free(&c[0]);
    uint32_t B = (uint32_t)std::sqrt((double)M);
    if (B < 1) B = 1;
    auto same = [&](kite_num *p, kite_num *q) {
        Giant a, b;
        pp_from_num(ctx, p, &a.g);
        pp_from_num(ctx, q, &b.g);
        return std::make_pair(giants_equal(a.g, b.g), pp_res64(&a.g));
    };
    int rc = -1;
    // x_{t+1} = x_t^(2^B), d = prod of the x_{jB}; d_T == d_{T-1}^(2^B) * x_0 checks the blocks,
    // a doubled tail the rest; up to three attempts
    for (int attempt = 0; attempt < 3 && rc; attempt++) {
        kite_reset_roundoff(ctx);
        kite_copy(ctx, x, x0);
        kite_copy(ctx, d, x0);
        const uint32_t blocks = (uint32_t)M / B;
        for (uint32_t b = 0; b < blocks; b++) {
            if (b + 1 == blocks) kite_copy(ctx, e, d);
            kite_square_n(ctx, x, B);
            kite_mul(ctx, d, x);
        }
        if (blocks) {
            kite_square_n(ctx, e, B);
            kite_mul(ctx, e, x0);
            if (!same(d, e).first) continue;
        }
        const uint32_t tail = (uint32_t)M - blocks * B;
        kite_copy(ctx, e, x);
        kite_square_n(ctx, x, tail);
        kite_square_n(ctx, e, tail);
        const auto r = same(x, e);
        if (r.first && roundoff_ok(ctx)) {
            *cert_res64 = r.second;
            rc = 0;
        }
    }
    if (Mout) *Mout = (uint32_t)M;
    return rc;
}

}  // extern "C"
