// PRST-compatible Fermat proofs (include/kite_proof.h): the products, the certificate and its
// verification, on the GB300 engine.
//
// The proof is Pietrzak's verifiable-delay-function proof in the form PRST 14.1 uses for
// k*2^n - 1 (its src/proof.cpp; the reference restates it in src/prstproof.c:231-666).  A Fermat
// test x_{i+1} = x_i^2 from x_0 = a^k leaves count+1 = 2^t+1 points x_{pos[j]}.  Level i of the
// proof combines the 2^i points at odd multiples of count/2^(i+1) into one product D_i; the
// level's challenge h_i is a hash of the running value Y (at first the last point) and D_i, and
// Y <- Y * D_i^h_i.  The certificate applies the same challenges to x_0, and its verification
// squares the certificate M times and must land on Y.
//
// How it runs here.  A level's product is the root of a binary tree over its points in order,
// each inner node left^h * right with the challenge of its height (h_{i-1} just above the
// points, h_0 at the root).  The points of a level are all read into device numbers first and
// the tree is reduced height by height on the GPU (the reference walks the points one at a time
// with a stack of partial products; the products are the same residues, so the files are the
// same bytes).  Equalities are decided on the device (kite_equal_internal).  The roots-of-unity
// condition raises R = a^(N-1) once to the product of all its prime-power orders.  The
// certificate check is a Gerbicz-checked chain of squarings with rollback.  Files, hashes and
// challenges are host work.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kite_proof.h"
#include "drivers.h"
#include "layout.h"
#include "md5.h"

namespace {

using kd::Number;
using u128 = unsigned __int128;

constexpr double kRoundoffLimit = 0.40;

// ---- values -------------------------------------------------------------------------------

// A giant that frees its words.
struct OwnedGiant {
    pp_giant g{nullptr, 0};
    OwnedGiant() = default;
    OwnedGiant(const OwnedGiant &) = delete;
    OwnedGiant &operator=(const OwnedGiant &) = delete;
    ~OwnedGiant() { pp_giant_free(&g); }
};

std::vector<uint64_t> limbs_from_giant(const pp_giant &g, size_t nl) {
    std::vector<uint64_t> l(nl, 0);
    for (int32_t i = 0; i < g.len && (size_t)(i / 2) < nl; i++) l[i / 2] |= (uint64_t)g.w[i] << (i % 2 ? 32 : 0);
    return l;
}

// The little-endian bytes of a giant's words: the form files and challenges use.
std::vector<uint8_t> giant_bytes(const pp_giant &g) {
    std::vector<uint8_t> b((size_t)4 * (g.len > 0 ? g.len : 0));
    for (int32_t i = 0; i < g.len; i++)
        for (int s = 0; s < 4; s++) b[4 * (size_t)i + s] = (uint8_t)(g.w[i] >> (8 * s));
    return b;
}

std::string state_path(const char *prefix, const char *kind, int index) {
    return std::string(prefix) + "." + kind + "." + std::to_string(index);
}

void remove_state(const std::string &path) {
    std::remove(path.c_str());
    std::remove((path + ".md5").c_str());
}

// Reads the single value of <prefix>.<kind>.<index> into x; the file must carry iteration
// `expect`.  Prints which file is missing or corrupt otherwise.
bool load_value(kite_ctx *ctx, const char *prefix, const char *kind, int index, int type, uint32_t fp,
                int32_t expect, kite_num *x, OwnedGiant *keep = nullptr) {
    const std::string path = state_path(prefix, kind, index);
    OwnedGiant tmp;
    OwnedGiant &g = keep ? *keep : tmp;
    int32_t it = 0;
    if (pp_read(path.c_str(), type, fp, &it, &g.g, 1) != 0 || it != expect) {
        std::fprintf(stderr, "%s is missing or corrupt.\n", path.c_str());
        return false;
    }
    pp_to_num(ctx, &g.g, x);
    return true;
}

// ---- challenges -----------------------------------------------------------------------------

// The primes below 1000, once.
const std::vector<uint32_t> &small_primes() {
    static const std::vector<uint32_t> primes = [] {
        std::vector<bool> composite(1000, false);
        std::vector<uint32_t> v;
        for (uint32_t p = 2; p < 1000; p++) {
            if (composite[p]) continue;
            v.push_back(p);
            for (uint32_t q = p * p; q < 1000; q += p) composite[q] = true;
        }
        return v;
    }();
    return primes;
}

// The challenge of a level: MD5(fp || Y || D); its first two little-endian words, the low one
// made odd and the high one non-zero, form a 64-bit number that is then stepped by 2 until no
// prime below 1000 divides it (PRST proof.cpp hash_giants and make_prime).
u128 challenge(uint32_t fp, const pp_giant &Y, const pp_giant &D) {
    kg::Md5 m;
    const uint8_t f[4] = {(uint8_t)fp, (uint8_t)(fp >> 8), (uint8_t)(fp >> 16), (uint8_t)(fp >> 24)};
    m.update(f, 4);
    for (const pp_giant *g : {&Y, &D}) {
        const std::vector<uint8_t> b = giant_bytes(*g);
        if (!b.empty()) m.update(b.data(), b.size());
    }
    uint8_t d[16];
    m.digest(d);
    uint32_t w[2];
    for (int i = 0; i < 2; i++)
        w[i] = (uint32_t)d[4 * i] | (uint32_t)d[4 * i + 1] << 8 | (uint32_t)d[4 * i + 2] << 16 |
               (uint32_t)d[4 * i + 3] << 24;
    u128 c = (u128)(w[1] ? w[1] : 1) << 32 | (w[0] | 1u);
    auto has_small_factor = [&](u128 v) {
        for (uint32_t p : small_primes())
            if (v % p == 0) return true;
        return false;
    };
    while (has_small_factor(c)) c += 2;
    return c;
}

u128 challenge_of(kite_ctx *ctx, uint32_t fp, const kite_num *Y, const pp_giant &D) {
    OwnedGiant y;
    pp_from_num(ctx, Y, &y.g);
    return challenge(fp, y.g, D);
}

// ---- arithmetic on the device ----------------------------------------------------------------

// out = base^e for e >= 1 (left-to-right binary powering); out and base are distinct numbers.
void raise(kite_ctx *ctx, kite_num *out, const kite_num *base, u128 e) {
    int top = 127;
    while (top > 0 && !((e >> top) & 1)) top--;
    kite_copy(ctx, out, base);
    for (int b = top - 1; b >= 0; b--) {
        kite_square(ctx, out);
        if ((e >> b) & 1) kite_mul(ctx, out, base);
    }
}

// The same with an exponent of any size, given as 64-bit words (least significant first).
void raise_big(kite_ctx *ctx, kite_num *out, const kite_num *base, const std::vector<uint64_t> &e) {
    int64_t top = (int64_t)e.size() * 64 - 1;
    while (top > 0 && !((e[top / 64] >> (top % 64)) & 1)) top--;
    kite_copy(ctx, out, base);
    for (int64_t b = top - 1; b >= 0; b--) {
        kite_square(ctx, out);
        if ((e[b / 64] >> (b % 64)) & 1) kite_mul(ctx, out, base);
    }
}

bool roundoff_ok(kite_ctx *ctx) { return kite_max_roundoff(ctx) < kRoundoffLimit; }

int levels_of(int count) {
    int t = 0;
    while ((1 << t) < count) t++;
    return t;
}

// ---- roots of unity ---------------------------------------------------------------------------

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

// (N - 1) mod m = (k*2^n - 2) mod m
uint64_t nm1_mod(uint64_t k, uint64_t n, uint64_t m) {
    uint64_t pow2 = 1 % m, sq = 2 % m;
    for (uint64_t e = n; e; e >>= 1, sq = mulmod(sq, sq, m))
        if (e & 1) pow2 = mulmod(pow2, sq, m);
    return (mulmod(k % m, pow2, m) + 2 * m - 2 % m) % m;
}

// PRST's condition on a composite result (its proof.cpp:82 at security 24): R = a^(N-1) must not
// be a root of unity of order dividing E = 2 * prod d_p, where d_p is the largest power below
// 2^31 of each odd prime p < 2^12 that divides N - 1 (N - 1 = 2(k 2^(n-1) - 1) holds 2 once).
// R^E is formed in one powering by E.  `xn` is the last point, a^(N+1).  A probable prime, or a
// base whose primes make up too much of N, passes unchecked.  true when the condition holds.
bool roots_of_unity_ok(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, const pp_giant &xn) {
    const size_t nl = kite_limbs(ctx);
    std::vector<uint64_t> r = limbs_from_giant(xn, nl);
    if (kg::residue_nm1(r.data(), ctx->lay.Nl.data(), nl, a) != 0) return true;
    if (kd::limbs_equal_word(r, 1)) return true;
    std::vector<uint64_t> E{2};  // the exponent, as a growing multi-word integer
    auto times = [&](uint64_t f) {
        u128 carry = 0;
        for (uint64_t &w : E) {
            carry += (u128)w * f;
            w = (uint64_t)carry;
            carry >>= 64;
        }
        if (carry) E.push_back((uint64_t)carry);
    };
    for (uint32_t p = 3; p < 4096; p += 2) {
        bool prime = true;
        for (uint32_t q = 3; q * q <= p && prime; q += 2) prime = p % q != 0;
        if (!prime || nm1_mod(k, n, p) != 0) continue;
        uint64_t d = p;
        while (d * p < 2147483647u && nm1_mod(k, n, d * p) == 0) d *= p;
        times(d);
    }
    Number R(ctx), X(ctx), one(ctx);
    kite_set_limbs(ctx, R, r.data());
    raise_big(ctx, X, R, E);
    kite_set_u64(ctx, one, 1);
    return kite_equal_internal(ctx, X, one) == 0;
}

// ---- the certificate's check: x <- x^(2^count), Gerbicz-checked -------------------------------

// Blocks of B squarings with d <- d*x; after each quarter of the blocks the identity
// d == x0 * t^(2^B) (t = d before the last update) is checked on the device and the state kept as
// verified, or restored from the last verified one (at most `tries` failures in all).  The
// count mod B squarings after the blocks are done twice and compared.
bool checked_power_of_two(kite_ctx *ctx, kite_num *x, uint64_t count, uint32_t B, int tries) {
    Number x0(ctx), d(ctx), t(ctx), vx(ctx), vd(ctx);
    kite_copy(ctx, x0, x);
    kite_copy(ctx, d, x);
    kite_copy(ctx, vx, x);
    kite_copy(ctx, vd, x);
    const uint64_t blocks = count / B;
    const uint64_t per_check = std::max<uint64_t>(1, (blocks + 3) / 4);
    uint64_t verified = 0;
    int failures = 0;
    while (verified < blocks) {
        const uint64_t upto = std::min(blocks, verified + per_check);
        for (uint64_t done = verified; done < upto; done++) {
            kite_copy(ctx, t, d);
            kite_square_n(ctx, x, B);
            kite_mul(ctx, d, x);
        }
        kite_square_n(ctx, t, B);
        kite_mul(ctx, t, x0);
        if (roundoff_ok(ctx) && kite_equal_internal(ctx, t, d) == 1) {
            kite_copy(ctx, vx, x);
            kite_copy(ctx, vd, d);
            verified = upto;
            continue;
        }
        if (++failures >= tries) return false;
        kite_copy(ctx, x, vx);
        kite_copy(ctx, d, vd);
    }
    const uint64_t tail = count - blocks * B;
    for (;;) {
        kite_copy(ctx, t, x);
        kite_square_n(ctx, x, tail);
        kite_square_n(ctx, t, tail);
        if (roundoff_ok(ctx) && kite_equal_internal(ctx, x, t) == 1) return true;
        if (++failures >= tries) return false;
        kite_copy(ctx, x, vx);
    }
}

}  // namespace

extern "C" {

void pp_from_num(kite_ctx *ctx, const kite_num *x, pp_giant *g) {
    const std::vector<uint64_t> l = kd::limbs_of(ctx, x);
    int32_t len = (int32_t)(2 * l.size());
    auto word = [&](int32_t i) { return (uint32_t)(l[i / 2] >> (i % 2 ? 32 : 0)); };
    while (len > 0 && word(len - 1) == 0) len--;
    g->w = static_cast<uint32_t *>(std::malloc(4 * (size_t)len + 4));
    g->len = len;
    for (int32_t i = 0; i < len; i++) g->w[i] = word(i);
}

void pp_to_num(kite_ctx *ctx, const pp_giant *g, kite_num *x) {
    const std::vector<uint64_t> l = limbs_from_giant(*g, kite_limbs(ctx));
    kite_set_limbs(ctx, x, l.data());
}

int pp_save_products(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count, const char *prefix, int keep,
                     volatile int *abort_flag, uint64_t *raw_res64) {
    const uint32_t fpN = pp_fingerprint(k, n), fpP = pp_proof_fingerprint(k, n, a);
    const int t = levels_of(count);
    std::vector<uint32_t> pos(count + 1);
    pp_points((uint32_t)n, count, pos.data());
    std::vector<u128> h(t, 0);
    Number Y(ctx), D(ctx), T(ctx);
    kite_reset_roundoff(ctx);
    if (!load_value(ctx, prefix, "proof", count, PP_TYPE_VALUE, fpP, (int32_t)pos[count], Y)) return -1;
    auto stopped = [&] { return abort_flag && *abort_flag; };
    // Y <- Y * D^h with h = challenge(Y, D)
    auto absorb = [&](int level, const pp_giant &dg) {
        h[level] = challenge_of(ctx, fpN, Y, dg);
        raise(ctx, T, D, h[level]);
        kite_mul(ctx, Y, T);
    };
    // products an interrupted run left: one powering each, nothing redone
    int level = 0;
    for (; level < t; level++) {
        OwnedGiant dg;
        int32_t it = -1;
        const std::string path = state_path(prefix, "prod", level);
        if (pp_read(path.c_str(), PP_TYPE_PRODUCT, fpP, &it, &dg.g, 1) != 0 || it != level) break;
        pp_to_num(ctx, &dg.g, D);
        absorb(level, dg.g);
    }
    for (; level < t; level++) {
        if (stopped()) return PP_ABORTED;
        // the level's points, in order, into device numbers
        const int width = 1 << level, stride = count >> level;  // points at odd multiples of stride/2
        std::vector<Number> nodes;
        nodes.reserve(width);
        for (int j = 0; j < width; j++) {
            if (stopped()) return PP_ABORTED;
            const int idx = stride / 2 + j * stride;
            nodes.emplace_back(ctx);
            if (!load_value(ctx, prefix, "proof", idx, PP_TYPE_VALUE, fpP, (int32_t)pos[idx], nodes.back())) return -1;
        }
        // reduce height by height: node <- left^h * right, h_{level-1} first, h_0 at the root
        for (int height = 1; height <= level; height++) {
            const u128 e = h[level - height];
            const int span = 1 << height;
            for (int j = 0; j < width; j += span) {
                kite_num *left = nodes[j], *right = nodes[j + span / 2];
                raise(ctx, T, left, e);
                kite_mul(ctx, T, right);
                kite_copy(ctx, left, T);
            }
        }
        kite_copy(ctx, D, nodes[0]);
        nodes.clear();
        OwnedGiant dg;
        pp_from_num(ctx, D, &dg.g);
        const std::string path = state_path(prefix, "prod", level);
        if (pp_write(path.c_str(), PP_TYPE_PRODUCT, fpP, level, &dg.g, 1)) {
            std::fprintf(stderr, "Write to %s failed.\n", path.c_str());
            return -1;
        }
        absorb(level, dg.g);
        if (!roundoff_ok(ctx)) {
            std::fprintf(stderr, "round-off error while compressing proof points.\n");
            return -1;
        }
    }
    {
        OwnedGiant yg;
        pp_from_num(ctx, Y, &yg.g);
        *raw_res64 = pp_res64(&yg.g);
    }
    if (!keep)
        for (int i = 1; i < count; i++) remove_state(state_path(prefix, "proof", i));
    return 0;
}

int pp_build_cert(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count, const char *prefix, int keep,
                  uint64_t *cert_res64) {
    const uint32_t fpN = pp_fingerprint(k, n), fpP = pp_proof_fingerprint(k, n, a);
    const int t = levels_of(count);
    std::vector<uint32_t> pos(count + 1);
    pp_points((uint32_t)n, count, pos.data());
    Number X(ctx), Y(ctx), D(ctx), T(ctx);
    kite_reset_roundoff(ctx);
    // point 0 must be a^k
    if (!load_value(ctx, prefix, "proof", 0, PP_TYPE_VALUE, fpP, 0, X)) return -1;
    kd::power_of_base(ctx, T, k, a, n);
    if (kite_equal_internal(ctx, X, T) != 1) {
        std::fprintf(stderr, "invalid a^k.\n");
        return -1;
    }
    {
        OwnedGiant last;
        if (!load_value(ctx, prefix, "proof", count, PP_TYPE_VALUE, fpP, (int32_t)pos[count], Y, &last)) return -1;
        if (!roots_of_unity_ok(ctx, k, n, a, last.g)) {
            std::fprintf(stderr, "roots of unity check failed.\n");
            return -1;
        }
    }
    // per level: X <- X^(h b) * D (b = 2 when the span M is odd), Y <- Y * D^h, M <- M / 2
    uint32_t M = pos[count];
    for (int level = 0; level < t; level++, M >>= 1) {
        OwnedGiant dg;
        if (!load_value(ctx, prefix, "prod", level, PP_TYPE_PRODUCT, fpP, level, D, &dg)) return -1;
        const u128 hl = challenge_of(ctx, fpN, Y, dg.g);
        raise(ctx, T, X, hl * (M & 1 ? 2 : 1));
        kite_mul(ctx, T, D);
        kite_copy(ctx, X, T);
        raise(ctx, T, D, hl);
        kite_mul(ctx, Y, T);
        if (!roundoff_ok(ctx)) {
            std::fprintf(stderr, "round-off error while building the certificate.\n");
            return -1;
        }
    }
    OwnedGiant yg;
    pp_from_num(ctx, Y, &yg.g);
    if (yg.g.len == 0) {
        std::fprintf(stderr, "invalid proof, the certificate is zero.\n");
        return -1;
    }
    *cert_res64 = pp_res64(&yg.g);
    // the certificate: X, then the empty a_power and a_base of a smooth test
    pp_giant cert[3] = {{nullptr, 0}, {nullptr, 0}, {nullptr, 0}};
    pp_from_num(ctx, X, &cert[0]);
    const std::string path = std::string(prefix) + ".cert";
    const int w = pp_write(path.c_str(), PP_TYPE_CERT, fpN, (int32_t)M, cert, 3);
    pp_giant_free(&cert[0]);
    if (w) {
        std::fprintf(stderr, "Write to %s failed.\n", path.c_str());
        return -1;
    }
    if (!keep) {
        remove_state(state_path(prefix, "proof", 0));
        remove_state(state_path(prefix, "proof", count));
        for (int level = 0; level < t; level++) remove_state(state_path(prefix, "prod", level));
    }
    return 0;
}

int pp_verify_cert(kite_ctx *ctx, uint64_t k, uint64_t n, const char *path, uint64_t *cert_res64, uint32_t *Mout) {
    pp_giant c[3];
    int32_t M = -1;
    const bool read = pp_read(path, PP_TYPE_CERT, pp_fingerprint(k, n), &M, c, 3) == 0;
    if (!read || M < 0) {
        for (pp_giant &g : c)
            if (read) pp_giant_free(&g);
        std::fprintf(stderr, "Invalid certificate file.\n");
        return -1;
    }
    const bool li = c[1].len != 0;  // Gerbicz-Li certificates come from tests of other forms
    pp_giant_free(&c[1]);
    pp_giant_free(&c[2]);
    if (li) {
        pp_giant_free(&c[0]);
        std::fprintf(stderr, "Gerbicz-Li certificates are not supported.\n");
        return -1;
    }
    Number x(ctx);
    pp_to_num(ctx, &c[0], x);
    pp_giant_free(&c[0]);
    kite_reset_roundoff(ctx);
    const uint32_t B = std::max<uint32_t>(1, (uint32_t)std::sqrt((double)M));
    if (Mout) *Mout = (uint32_t)M;
    if (!checked_power_of_two(ctx, x, (uint64_t)M, B, 3)) return -1;
    OwnedGiant g;
    pp_from_num(ctx, x, &g.g);
    *cert_res64 = pp_res64(&g.g);
    return 0;
}

}  // extern "C"
