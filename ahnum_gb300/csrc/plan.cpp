// Per-FFT-length plans (see plan.h).
#include "plan.h"

#include <cuda_runtime.h>

#include <cstdlib>

#include "../../include/kite_cuda.h"

#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>

namespace kg {

LengthPlan::~LengthPlan() {
    if (device < 0) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaFree(twr);
    cudaFree(twc);
    cudaFree(t4);
    cudaFree(sw);
    cudaFree(dposr);
    cudaFree(dposc);
    cudaFree(dpairs);
    if (prev >= 0) cudaSetDevice(prev);
}

static bool factorable(uint32_t n) {
    for (uint32_t p : {2u, 3u, 5u, 7u})
        while (n % p == 0) n /= p;
    return n == 1;
}

static bool shape_usable(uint32_t H, uint32_t r, uint32_t c) {
    return r >= 2 && r <= 1024 && c >= 16 && c <= 2048 && c % kGroup == 0 && (uint64_t)r * c == H &&
           factorable(r) && factorable(c);
}

// Shapes chosen by the autotuner (or a tuning file), by FFT length L = 2H: R rows.
static std::mutex g_shape_mu;
static std::map<uint32_t, uint32_t> g_shape;

bool set_shape_override(uint32_t L, uint32_t R) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    if (!R) {
        g_shape.erase(L);
        return true;
    }
    if (L % 2 || R == 0 || (L / 2) % R || !shape_usable(L / 2, R, L / 2 / R)) return false;
    g_shape[L] = R;
    return true;
}

int shape_candidates(uint32_t H, uint32_t *R, uint32_t *C, int max) {
    int n = 0;
    for (uint32_t c = 16; c <= 2048 && c <= H / 2 && n < max; c += kGroup) {
        if (H % c || !shape_usable(H, H / c, c)) continue;
        const double ratio = (double)c / (H / c);
        if (ratio < 0.5 || ratio > 64) continue;  // far from balanced: never the fastest
        R[n] = H / c;
        C[n] = c;
        n++;
    }
    return n;
}

bool choose_shape(uint32_t H, uint32_t &R, uint32_t &C) {
    static std::once_flag env_once;
    std::call_once(env_once, [] {
        if (const char *p = std::getenv("KITE_GB300_TUNING")) kc_tuning_load(p);
    });
    {
        std::lock_guard<std::mutex> lock(g_shape_mu);
        auto it = g_shape.find(2 * H);
        if (it != g_shape.end()) {
            R = it->second;
            C = H / R;
            return true;
        }
    }
    double best = 1e30;
    R = C = 0;
    // rows up to 2048 points: a product's row pass holds 6 rows of C points in shared memory
    for (uint32_t c = 16; c <= 2048 && c <= H / 2; c += kGroup) {
        if (H % c) continue;
        uint32_t r = H / c;
        if (!shape_usable(H, r, c)) continue;
        // rows about four times as long as columns
        double cost = std::fabs(std::log2((double)r) - std::log2((double)c) + 2.0);
        if (cost < best) {
            best = cost;
            R = r;
            C = c;
        }
    }
    return R != 0;
}

static int radix_stages(uint32_t n) {
    int st = 0;
    for (; n % 4 == 0; n /= 4) st++;
    for (uint32_t p : {2u, 3u, 5u, 7u})
        for (; n % p == 0; n /= p) st++;
    return st;
}

// Latency shapes chosen by the autotuner (or a tuning file), by FFT length L = 2H: (R, G).
static std::map<uint32_t, std::pair<uint32_t, int>> g_latency;

// the carry into a segment must be absorbed by 2g-1 digits of at least min_bits (a product's
// carry stays below 2^(51 - b)), and the top region must fit one segment
static bool group_fits(int g, unsigned min_bits, unsigned top_digits) {
    return (2 * g - 1) * (int)min_bits >= 51 - (int)min_bits && (int)top_digits <= 2 * g;
}

bool set_latency_override(uint32_t L, uint32_t R, int G) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    if (!R) {
        g_latency.erase(L);
        return true;
    }
    if (L % 2 || (L / 2) % R || !shape_usable(L / 2, R, L / 2 / R) || (G != 2 && G != 4 && G != 8) ||
        (L / 2 / R) % G)
        return false;
    g_latency[L] = {R, G};
    return true;
}

bool choose_latency_shape(uint32_t H, int nsm, unsigned min_bits, unsigned top_digits, uint32_t &R,
                          uint32_t &C, int &G) {
    {
        // an autotuned shape of this length, where this number's digits allow its groups
        std::lock_guard<std::mutex> lock(g_shape_mu);
        auto it = g_latency.find(2 * H);
        if (it != g_latency.end() && group_fits(it->second.second, min_bits, top_digits)) {
            R = it->second.first;
            C = H / R;
            G = it->second.second;
            return true;
        }
    }
    // FP64 lane-operations per point of each pass (measured: rows ~53, each column pass ~24),
    // a fixed cost per stage barrier, and the load of the busiest SM.
    double best = 1e300;
    R = C = 0;
    G = kGroup;
    if (nsm < 1) nsm = 1;
    for (uint32_t c = 16; c <= 2048 && c <= H / 2; c += kGroup) {
        if (H % c || !shape_usable(H, H / c, c)) continue;
        const uint32_t r = H / c;
        for (int g : {2, 4, 8}) {
            if (!group_fits(g, min_bits, top_digits)) continue;
            const double pairs = r / 2 + 1, groups = c / g;
            const double rows = std::ceil(pairs / nsm) * 106.0 * c + 800.0 * (2 * radix_stages(c) + 2);
            const double cols = std::ceil(groups / nsm) * 24.0 * r * g + 800.0 * (radix_stages(r) + 2);
            const double cost = rows + 2 * cols;
            if (cost < best - 1e-9) {
                best = cost;
                R = r;
                C = c;
                G = g;
            }
        }
    }
    return R != 0;
}

bool make_fft_plan(int n, FftPlan &pl) {
    // radix 4 throughout the power-of-two part (tangent twiddles), one radix 2 if needed, and
    // the odd radices last: the last plan stage has span 1 and runs without twiddles, so the
    // costlier odd butterflies take no twiddle multiplications there.
    pl = FftPlan{};
    pl.n = n;
    int m = n, st = 0;
    auto push = [&](int p) {
        if (st >= kMaxStages) return false;
        pl.rad[st++] = p;
        m /= p;
        return true;
    };
    while (m % 4 == 0)
        if (!push(4)) return false;
    if (m % 2 == 0 && !push(2)) return false;
    for (int p : {3, 5, 7})
        while (m % p == 0)
            if (!push(p)) return false;
    if (m != 1) return false;
    pl.nst = st;
    int span = n, off = 0;
    for (int i = 0; i < st; i++) {
        span /= pl.rad[i];
        pl.span[i] = span;
        pl.off[i] = off;
        off += (pl.rad[i] - 1) * span;
    }
    return true;
}

double2 cis_neg(uint64_t j, uint64_t m) {
    j %= m;
    // angle pi*x with x = num/den = 2j/m in [0, 2), reduced to [0, 1/4] by exact reflections
    uint64_t num = 2 * j, den = m;
    double sc = 1, ss = 1;
    bool swap = false;
    if (num > den) {  // cos(pi x) = -cos(pi(x-1)), sin likewise
        num -= den;
        sc = -sc;
        ss = -ss;
    }
    if (2 * num > den) {  // x -> 1 - x: cos negates
        num = den - num;
        sc = -sc;
    }
    if (4 * num > den) {  // x -> 1/2 - x: cos and sin swap
        num = den - 2 * num;
        den *= 2;
        swap = true;
    }
    long double th = 3.14159265358979323846264338327950288L * (long double)num / (long double)den;
    double c = (double)cosl(th), s = (double)sinl(th);
    if (swap) std::swap(c, s);
    return make_double2(sc * c, -ss * s);
}

static void positions(const FftPlan &pl, std::vector<int> &rev, std::vector<int> &pos) {
    int n = pl.n;
    rev.assign(n, 0);
    pos.assign(n, 0);
    for (int k = 0; k < n; k++) {
        int kk = k, p = 0;
        for (int i = 0; i < pl.nst; i++) {
            p += (kk % pl.rad[i]) * pl.span[i];
            kk /= pl.rad[i];
        }
        pos[k] = p;
        rev[p] = k;
    }
}

// Twiddle records of every stage (see FftPlan): tangent form for radix 2 and 4, complex
// twiddles for the odd radices.  A cosine that is exactly 0 is replaced by 2^-60 (and the
// tangent scaled to match), which changes the product by far less than one ulp.
static void stage_twiddles(const FftPlan &pl, std::vector<double2> &tw) {
    tw.clear();
    const double tiny = std::ldexp(1.0, -60);
    for (int i = 0; i < pl.nst; i++) {
        const int p = pl.rad[i], s = pl.span[i], sz = p * s;
        for (int j = 0; j < s; j++) {
            double c[4] = {1, 1, 1, 1}, tau[4] = {0, 0, 0, 0};
            double2 w[8];
            for (int t = 1; t < p; t++) {
                w[t] = cis_neg((uint64_t)t * j, (uint64_t)sz);
                double cc = w[t].x;
                if (cc == 0.0) cc = tiny;
                if (t < 4) {
                    c[t] = cc;
                    tau[t] = w[t].y / cc;
                }
            }
            if (p == 2) {
                tw.push_back(make_double2(tau[1], c[1]));
            } else if (p == 4) {
                tw.push_back(make_double2(tau[1], tau[2]));
                tw.push_back(make_double2(tau[3], c[1]));
                tw.push_back(make_double2(c[2], c[3] / c[1]));
            } else {
                for (int t = 1; t < p; t++) tw.push_back(w[t]);
            }
        }
    }
}

std::shared_ptr<LengthPlan> build_plan_host(uint32_t L, uint32_t rows, std::vector<double2> *twr,
                                            std::vector<double2> *twc, std::vector<double2> *t4,
                                            std::vector<double2> *sw) {
    if (L % (2 * kGroup) || L < 64) return nullptr;
    auto pl = std::make_shared<LengthPlan>();
    pl->L = L;
    pl->H = L / 2;
    if (rows) {
        if (pl->H % rows || !shape_usable(pl->H, rows, pl->H / rows)) return nullptr;
        pl->R = rows;
        pl->C = pl->H / rows;
    } else if (!choose_shape(pl->H, pl->R, pl->C)) {
        return nullptr;
    }
    if (!make_fft_plan((int)pl->C, pl->rp) || !make_fft_plan((int)pl->R, pl->cp)) return nullptr;
    positions(pl->rp, pl->rev_c, pl->pos_c);
    positions(pl->cp, pl->rev_r, pl->pos_r);
    const uint32_t R = pl->R, C = pl->C, H = pl->H;
    for (uint32_t kr = 0; kr < R; kr++) {
        uint32_t k2 = (R - kr) % R;
        if (kr <= k2) pl->pairs.push_back(make_int2((int)kr, (int)k2));
    }
    if (twr) stage_twiddles(pl->rp, *twr);
    if (twc) stage_twiddles(pl->cp, *twc);
    if (t4) {
        t4->resize((size_t)R * C);
        for (uint32_t kr = 0; kr < R; kr++)
            for (uint32_t c = 0; c < C; c++) (*t4)[(size_t)kr * C + c] = cis_neg((uint64_t)c * kr % H, H);
    }
    if (sw) {
        sw->resize((size_t)R * C);
        for (uint32_t kr = 0; kr < R; kr++)
            for (uint32_t kc = 0; kc < C; kc++)
                (*sw)[(size_t)kr * C + kc] = cis_neg(((uint64_t)kr + (uint64_t)R * kc) % H, H);
    }
    return pl;
}

template <class T>
static bool upload(const std::vector<T> &h, T **d, size_t &bytes) {
    size_t nb = h.size() * sizeof(T);
    if (cudaMalloc((void **)d, nb ? nb : sizeof(T)) != cudaSuccess) return false;
    bytes += nb;
    return !nb || cudaMemcpy(*d, h.data(), nb, cudaMemcpyHostToDevice) == cudaSuccess;
}

std::shared_ptr<LengthPlan> get_plan(uint32_t L, uint32_t R) {
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, uint32_t>, std::shared_ptr<LengthPlan>> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    uint32_t C = 0;
    if (L % 2 || (!R && !choose_shape(L / 2, R, C))) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({dev, L, R});
    if (it != cache.end()) return it->second;
    std::vector<double2> twr, twc, t4, sw;
    auto pl = build_plan_host(L, R, &twr, &twc, &t4, &sw);
    if (!pl) return nullptr;
    pl->device = dev;
    bool ok = upload(twr, &pl->twr, pl->device_bytes) && upload(twc, &pl->twc, pl->device_bytes) &&
              upload(t4, &pl->t4, pl->device_bytes) && upload(sw, &pl->sw, pl->device_bytes) &&
              upload(pl->pos_r, &pl->dposr, pl->device_bytes) && upload(pl->pos_c, &pl->dposc, pl->device_bytes) &&
              upload(pl->pairs, &pl->dpairs, pl->device_bytes);
    if (!ok) return nullptr;
    cache[{dev, L, R}] = pl;
    return pl;
}

}  // namespace kg
