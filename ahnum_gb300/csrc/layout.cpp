// Exact host-side arithmetic of the k-scaled IBDWT (see layout.h).
// Reference behaviour restated: src/ctx.c:17-221 (lengths, layout, weights), :345-407 (carry and
// fold), :409-559 (limbs), src/prp.c:63-144 (base^(N-1) residue).
#include "layout.h"

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

namespace kg {

using u128 = unsigned __int128;
using i128 = __int128;

// ---- FFT lengths (src/ctx.c:17-33, 94-148; no tuning file) ---------------------------------

bool fft_len_ok(uint32_t L) {
    if (L < 16 || (L & 1)) return false;
    for (uint32_t p : {2u, 3u, 5u, 7u})
        while (L % p == 0) L /= p;
    return L == 1;
}

double safe_bpw(uint32_t L, uint64_t k) {
    return 21.44 - 0.305 * (std::log2((double)L) - 12.0) - 0.5 * std::log2((double)k) - 0.2;
}

static double length_cost(uint32_t L) {
    double c = std::log2((double)L);
    uint32_t m = L;
    for (; m % 3 == 0; m /= 3) c += 0.6;
    for (; m % 5 == 0; m /= 5) c += 1.0;
    for (; m % 7 == 0; m /= 7) c += 1.4;
    return (double)L * c;
}

static bool length_usable(uint32_t L) { return L % 64 == 0 && fft_len_ok(L); }

// Measured microseconds per squaring by FFT length, from the autotuner or a tuning file; used as
// the reference uses its `kite tune` times (src/ctx.c:123-140).
static std::mutex g_times_mu;
static std::map<uint32_t, double> g_times;

void set_tuned_time(uint32_t L, double us) {
    std::lock_guard<std::mutex> lock(g_times_mu);
    if (us > 0) g_times[L] = us;
    else g_times.erase(L);
}

static double tuned_time(uint32_t L) {
    std::lock_guard<std::mutex> lock(g_times_mu);
    auto it = g_times.find(L);
    return it == g_times.end() ? -1.0 : it->second;
}

uint32_t choose_fft_len(uint64_t k, uint64_t n) {
    if (n < 2048) {
        for (uint32_t L = 16; L <= n; L *= 2)
            if ((double)n / L <= safe_bpw(L, k)) return L;
        return 0;
    }
    uint32_t lo = 0;
    for (uint32_t L = 64; L < (1u << 28); L += 64)
        if (length_usable(L) && (double)n / L <= safe_bpw(L, k)) {
            lo = L;
            break;
        }
    if (!lo) return 0;
    // among the usable lengths up to 30 % longer: the fastest measured one when every one of
    // them has a measurement, else the cheapest by the heuristic
    bool measured = true;
    for (uint32_t L = lo; L <= lo + lo / 10 * 3; L += 64)
        if (length_usable(L) && tuned_time(L) < 0) measured = false;
    uint32_t best = lo;
    double bc = HUGE_VAL;
    for (uint32_t L = lo; L <= lo + lo / 10 * 3; L += 64) {
        if (!length_usable(L)) continue;
        double c = measured ? tuned_time(L) : length_cost(L);
        if (c < bc) {
            bc = c;
            best = L;
        }
    }
    return best;
}

uint32_t next_fft_len(uint32_t L) {
    for (uint32_t M = (L / 64 + 1) * 64; M < (1u << 28); M += 64)
        if (fft_len_ok(M)) return M;
    return 0;
}

// ---- layout --------------------------------------------------------------------------------

// frac(log2 k) in 64 bits: square a 62-bit fixed-point mantissa 64 times, one result bit per
// square (the method of src/ctx.c:153-167, so the layout matches bit for bit).
static uint64_t log2_frac64(uint64_t k) {
    int e = 63 - __builtin_clzll(k);
    u128 y = (u128)k << (62 - e);
    uint64_t f = 0;
    for (int i = 0; i < 64; i++) {
        y = (y * y) >> 62;
        f <<= 1;
        if (y >> 63) {
            f |= 1;
            y >>= 1;
        }
    }
    return f;
}

bool Layout::build(uint64_t k_, uint64_t n_, uint32_t L_) {
    k = k_;
    n = n_;
    L = L_;
    if (!k || !(k & 1) || k >= (1ull << 30) || n < 8 || !fft_len_ok(L) || L > n) return false;
    lam = log2_frac64(k);
    const uint64_t e = (uint64_t)(63 - __builtin_clzll(k));
    const u128 tfix = ((u128)(n + e) << 64) + lam;  // T' * 2^64
    const u128 den = (u128)L << 64;
    s.assign((size_t)L + 1, 0);
    bits.assign(L, 0);
    w.assign(L, 0);
    oscale.assign(L, 0);
    for (uint32_t j = 0; j <= L; j++) s[j] = (uint64_t)(((u128)j * tfix + den - 1) / den);
    top_t = L;
    for (uint32_t j = 0; j < L; j++) {
        uint64_t b = s[j + 1] - s[j];
        if (b == 0 || b > 40) return false;
        bits[j] = (uint8_t)b;
        if (top_t == L && s[j + 1] > n) top_t = j;
        // exponent s_j - j T'/L = (s_j L 2^64 - j T' 2^64) / (L 2^64) in [0, 1); top 64 bits
        u128 num = (u128)s[j] * den - (u128)j * tfix;
        double frac = (double)(uint64_t)(num / L) / 18446744073709551616.0;
        w[j] = std::exp2(frac);
        oscale[j] = (double)k / w[j];
    }
    sL = s[L];
    top_st = top_t < L ? s[top_t] : sL;
    top_m = (uint32_t)(n - top_st);
    if (sL - top_st > 100 || top_t == 0) return false;
    nlimbs = (size_t)((n + 64 + 63) / 64);
    Nl.assign(nlimbs, 0);
    Nl[n / 64] = k << (n % 64);
    if (n % 64 && n / 64 + 1 < nlimbs) Nl[n / 64 + 1] = k >> (64 - n % 64);
    for (size_t i = 0; i < nlimbs; i++)
        if (Nl[i]--) break;
    return true;
}

// ---- carry and fold ------------------------------------------------------------------------

static inline int64_t balance_digit(int64_t v, unsigned b, int64_t &q) {
    q = (v + ((int64_t)1 << (b - 1))) >> b;  // arithmetic shift: floor
    return v - (q << b);
}

// Everything at or above 2^n -- top digits t..L-1 plus the carry cy at 2^{s_L} -- equals
// H*2^{s_t}; with m = n - s_t, H = lo + 2^m*hi and hi = q*k + r, k*2^n == 1 gives
// H*2^{s_t} == (lo + r 2^m)*2^{s_t} + q.  The region is re-centred to [-k 2^m/2, k 2^m/2) and
// q is returned for digit 0.
int64_t Layout::fold_top(int64_t *d, int64_t cy) const {
    i128 H = (i128)cy << (sL - top_st);
    unsigned pos = 0;
    for (uint32_t j = top_t; j < L; j++) {
        H += (i128)d[j] << pos;
        pos += bits[j];
    }
    const i128 K = (i128)k;
    i128 lo = H & (((i128)1 << top_m) - 1);
    i128 hi = H >> top_m;
    i128 q = hi / K;
    if (hi % K != 0 && hi < 0) q -= 1;
    i128 top = lo + ((hi - q * K) << top_m);
    const i128 span = K << top_m;
    if (2 * top >= span) {
        top -= span;
        q += 1;
    }
    for (uint32_t j = top_t; j + 1 < L; j++) {
        unsigned b = bits[j];
        i128 qq = (top + ((i128)1 << (b - 1))) >> b;
        d[j] = (int64_t)(top - (qq << b));
        top = qq;
    }
    if (top_t < L) d[L - 1] = (int64_t)top;
    return (int64_t)q;
}

void Layout::carry(int64_t *d) const {
    int64_t cy = 0;
    for (uint32_t j = 0; j < L; j++) d[j] = balance_digit(d[j] + cy, bits[j], cy);
    for (int pass = 0; pass < 64; pass++) {
        cy = fold_top(d, cy);
        for (uint32_t j = 0; j < top_t && cy; j++) d[j] = balance_digit(d[j] + cy, bits[j], cy);
        if (!cy) return;
        if (top_t < L) {  // the ripple reached the top region: fold again
            d[top_t] += cy;
            cy = 0;
        }
    }
}

// ---- limbs ---------------------------------------------------------------------------------

namespace {

void add_at(uint64_t *a, size_t na, uint64_t pos, uint64_t v) {
    size_t w = (size_t)(pos / 64);
    unsigned sh = (unsigned)(pos % 64);
    if (w >= na) return;
    u128 t = (u128)v << sh;
    u128 s = (u128)a[w] + (uint64_t)t;
    a[w] = (uint64_t)s;
    uint64_t c = (uint64_t)(s >> 64) + (uint64_t)(t >> 64);
    for (size_t i = w + 1; c && i < na; i++) {
        s = (u128)a[i] + c;
        a[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
}

int cmp(const uint64_t *a, const uint64_t *b, size_t n) {
    for (size_t i = n; i-- > 0;)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

void sub_in(uint64_t *a, const uint64_t *b, size_t n) {
    uint64_t br = 0;
    for (size_t i = 0; i < n; i++) {
        u128 d = (u128)a[i] - b[i] - br;
        a[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
}

void add_in(uint64_t *a, const uint64_t *b, size_t n) {
    uint64_t c = 0;
    for (size_t i = 0; i < n; i++) {
        u128 s = (u128)a[i] + b[i] + c;
        a[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
}

void mul_word(uint64_t *a, size_t n, uint64_t m) {
    u128 c = 0;
    for (size_t i = 0; i < n; i++) {
        c += (u128)a[i] * m;
        a[i] = (uint64_t)c;
        c >>= 64;
    }
}

uint64_t div_word(uint64_t *a, size_t n, uint64_t m) {
    u128 r = 0;
    for (size_t i = n; i-- > 0;) {
        r = (r << 64) | a[i];
        a[i] = (uint64_t)(r / m);
        r %= m;
    }
    return (uint64_t)r;
}

uint64_t mod_word(const uint64_t *a, size_t n, uint64_t m) {
    u128 r = 0;
    for (size_t i = n; i-- > 0;) r = ((r << 64) | a[i]) % m;
    return (uint64_t)r;
}

uint64_t get_bits(const uint64_t *a, size_t na, uint64_t pos, unsigned cnt) {
    size_t w = (size_t)(pos / 64);
    unsigned sh = (unsigned)(pos % 64);
    if (w >= na) return 0;
    u128 v = a[w];
    if (w + 1 < na) v |= (u128)a[w + 1] << 64;
    v >>= sh;
    return cnt >= 64 ? (uint64_t)v : (uint64_t)v & (((uint64_t)1 << cnt) - 1);
}

}  // namespace

// a (na limbs) -> a mod N in a[0..nlimbs), by a = lo + 2^n hi, hi = q k + r -> lo + r 2^n + q
void Layout::reduce_mod_N(uint64_t *a, size_t na) const {
    const size_t w0 = (size_t)(n / 64);
    const unsigned sh = (unsigned)(n % 64);
    const size_t nh = na - w0 + 1;
    std::vector<uint64_t> hi(nh);
    for (;;) {
        std::fill(hi.begin(), hi.end(), 0);
        for (size_t i = w0; i < na; i++) {
            size_t o = i - w0;
            hi[o] |= sh ? a[i] >> sh : a[i];
            if (sh && o) hi[o - 1] |= a[i] << (64 - sh);
        }
        bool small = hi[0] < k;
        for (size_t i = 1; i < nh && small; i++) small = hi[i] == 0;
        if (small) break;  // a < k 2^n = N + 1
        uint64_t r = div_word(hi.data(), nh, k);
        if (sh) a[w0] &= ((uint64_t)1 << sh) - 1;
        else a[w0] = 0;
        for (size_t i = w0 + 1; i < na; i++) a[i] = 0;
        add_at(a, na, n, r);
        for (size_t i = 0; i < nh; i++)
            if (hi[i]) add_at(a, na, 64 * (uint64_t)i, hi[i]);
    }
    if (cmp(a, Nl.data(), nlimbs) >= 0) sub_in(a, Nl.data(), nlimbs);
}

void Layout::digits_to_limbs(const int64_t *d, uint64_t *limbs) const {
    size_t na = (size_t)((sL + 64 + 40) / 64 + 3);
    if (na < nlimbs + 2) na = nlimbs + 2;
    std::vector<uint64_t> P(na), M(na);
    for (uint32_t j = 0; j < L; j++) {
        int64_t v = d[j];
        if (v > 0) add_at(P.data(), na, s[j], (uint64_t)v);
        else if (v < 0) add_at(M.data(), na, s[j], (uint64_t)(-(v + 1)) + 1);
    }
    // the stored value is x/k: x = k * V
    mul_word(P.data(), na, k);
    mul_word(M.data(), na, k);
    reduce_mod_N(P.data(), na);
    reduce_mod_N(M.data(), na);
    if (cmp(P.data(), M.data(), nlimbs) < 0) add_in(P.data(), Nl.data(), nlimbs);
    sub_in(P.data(), M.data(), nlimbs);
    std::memcpy(limbs, P.data(), nlimbs * sizeof(uint64_t));
}

void Layout::limbs_to_digits(const uint64_t *limbs, int64_t *d) const {
    const size_t na = nlimbs + 2;
    std::vector<uint64_t> a(na);
    std::memcpy(a.data(), limbs, nlimbs * sizeof(uint64_t));
    // x = q k + r  ->  x/k == x 2^n == q + r 2^n (mod N)
    uint64_t r = div_word(a.data(), na, k);
    add_at(a.data(), na, n, r);
    if (cmp(a.data(), Nl.data(), nlimbs) >= 0 && !a[nlimbs] && !a[nlimbs + 1])
        sub_in(a.data(), Nl.data(), nlimbs);
    for (uint32_t j = 0; j + 1 < L; j++) d[j] = (int64_t)get_bits(a.data(), na, s[j], bits[j]);
    d[L - 1] = (int64_t)get_bits(a.data(), na, s[L - 1], 64);
    carry(d);
}

int Layout::constant_digits(int64_t c, uint32_t *idx, int64_t *val, int cap) const {
    std::vector<uint64_t> l(nlimbs, 0);
    // limbs of c mod N
    if (c >= 0) {
        l[0] = (uint64_t)c;
    } else {
        std::memcpy(l.data(), Nl.data(), nlimbs * sizeof(uint64_t));
        std::vector<uint64_t> m(nlimbs, 0);
        m[0] = (uint64_t)(-c);
        sub_in(l.data(), m.data(), nlimbs);
    }
    std::vector<int64_t> d(L);
    limbs_to_digits(l.data(), d.data());
    int cnt = 0;
    for (uint32_t j = 0; j < L; j++) {
        if (!d[j]) continue;
        if (cnt == cap) return -1;
        idx[cnt] = j;
        val[cnt] = d[j];
        cnt++;
    }
    return cnt;
}

// ---- base^(N-1) ------------------------------------------------------------------------------

// a <- a / d mod m for a < m, gcd(d, m) = 1: add t*m so that d divides, then divide
static void divide_mod(uint64_t *a, const uint64_t *m, size_t n, uint64_t d) {
    uint64_t am = mod_word(a, n, d), mm = mod_word(m, n, d), t = 0;
    while ((am + (u128)t * mm) % d) t++;
    std::vector<uint64_t> acc(n + 1, 0), tm(n + 1, 0);
    std::memcpy(acc.data(), a, n * sizeof(uint64_t));
    std::memcpy(tm.data(), m, n * sizeof(uint64_t));
    mul_word(tm.data(), n + 1, t);
    add_in(acc.data(), tm.data(), n + 1);
    div_word(acc.data(), n + 1, d);
    std::memcpy(a, acc.data(), n * sizeof(uint64_t));
}

int residue_nm1(uint64_t *y, const uint64_t *N, size_t nl, uint64_t base) {
    uint64_t Q = 1, b = base;
    std::vector<uint64_t> M(N, N + nl);
    for (uint64_t p = 2; b > 1; p++) {
        if (b % p) continue;
        while (b % p == 0) b /= p;
        while (mod_word(M.data(), nl, p) == 0) {
            if (Q > (1ull << 40)) return -1;
            Q *= p;
            div_word(M.data(), nl, p);
        }
    }
    if (Q == 1) {
        divide_mod(y, N, nl, base);
        divide_mod(y, N, nl, base);
        return 0;
    }
    // x == 0 (mod Q), x == y / base^2 (mod M)
    // r = y mod M; y < N = Q M with Q < 2^41, so subtract M*2^b for b = 41..0
    std::vector<uint64_t> r(y, y + nl);
    r.push_back(0);
    for (int bit = 41; bit >= 0; bit--) {
        std::vector<uint64_t> mb(nl + 1, 0);
        for (size_t i = 0; i < nl; i++) {
            mb[i + bit / 64] |= M[i] << (bit % 64);
            if (bit % 64 && i + bit / 64 + 1 <= nl) mb[i + bit / 64 + 1] |= M[i] >> (64 - bit % 64);
        }
        if (cmp(r.data(), mb.data(), nl + 1) >= 0) sub_in(r.data(), mb.data(), nl + 1);
    }
    r.pop_back();
    divide_mod(r.data(), M.data(), nl, base);
    divide_mod(r.data(), M.data(), nl, base);
    uint64_t rm = mod_word(r.data(), nl, Q), mm = mod_word(M.data(), nl, Q), u = 0;
    while ((rm + (u128)mm * u) % Q) u++;
    std::vector<uint64_t> t(M);
    t.push_back(0);
    r.push_back(0);
    mul_word(t.data(), nl + 1, u);
    add_in(r.data(), t.data(), nl + 1);
    std::memcpy(y, r.data(), nl * sizeof(uint64_t));
    return 0;
}

}  // namespace kg
