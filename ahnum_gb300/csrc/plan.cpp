// Per-FFT-length plans (see plan.h).
#include "plan.h"

#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <mutex>
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
    cudaFree(part0);
    cudaFree(part1);
    cudaFree(dpairs);
    if (prev >= 0) cudaSetDevice(prev);
}

static bool factorable(uint32_t n) {
    for (uint32_t p : {2u, 3u, 5u, 7u})
        while (n % p == 0) n /= p;
    return n == 1;
}

bool choose_shape(uint32_t H, uint32_t &R, uint32_t &C) {
    double best = 1e30;
    R = C = 0;
    for (uint32_t c = 16; c <= 4096 && c <= H / 2; c += kGroup) {
        if (H % c) continue;
        uint32_t r = H / c;
        if (r < 2 || r > 2048 || !factorable(r) || !factorable(c)) continue;
        // rows about four times as long as columns; columns beyond 1024 points need more
        // shared memory per group than a CTA should hold
        double cost = std::fabs(std::log2((double)r) - std::log2((double)c) + 2.0);
        if (r > 1024) cost += 10;
        if (cost < best) {
            best = cost;
            R = r;
            C = c;
        }
    }
    return R != 0;
}

bool make_fft_plan(int n, FftPlan &pl) {
    pl = FftPlan{};
    pl.n = n;
    int m = n, st = 0;
    auto push = [&](int p) {
        if (st >= kMaxStages) return false;
        pl.rad[st++] = p;
        m /= p;
        return true;
    };
    while (m % 8 == 0 && m > 8)
        if (!push(8)) return false;
    for (int p : {8, 4, 2, 3, 5, 7})
        while (m % p == 0)
            if (!push(p)) return false;
    if (m != 1) return false;
    pl.nst = st;
    int span = n, off = 0;
    for (int i = 0; i < st; i++) {
        span /= pl.rad[i];
        pl.span[i] = span;
        pl.off[i] = off;
        off += pl.rad[i] * span;
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

static void stage_twiddles(const FftPlan &pl, std::vector<double2> &tw) {
    tw.clear();
    for (int i = 0; i < pl.nst; i++) {
        int p = pl.rad[i], s = pl.span[i], sz = p * s;
        for (int t = 0; t < p; t++)
            for (int j = 0; j < s; j++) tw.push_back(cis_neg((uint64_t)t * j, (uint64_t)sz));
    }
}

std::shared_ptr<LengthPlan> build_plan_host(uint32_t L, std::vector<double2> *twr,
                                            std::vector<double2> *twc, std::vector<double2> *t4,
                                            std::vector<double2> *sw, std::vector<int> *part0,
                                            std::vector<int> *part1) {
    if (L % (2 * kGroup) || L < 64) return nullptr;
    auto pl = std::make_shared<LengthPlan>();
    pl->L = L;
    pl->H = L / 2;
    if (!choose_shape(pl->H, pl->R, pl->C)) return nullptr;
    pl->NG = pl->C / kGroup;
    if (!make_fft_plan((int)pl->C, pl->rp) || !make_fft_plan((int)pl->R, pl->cp)) return nullptr;
    positions(pl->rp, pl->rev_c, pl->pos_c);
    positions(pl->cp, pl->rev_r, pl->pos_r);
    const uint32_t R = pl->R, C = pl->C, H = pl->H;
    for (uint32_t p = 0; p < R; p++) {
        int kr = pl->rev_r[p];
        int p2 = pl->pos_r[(R - kr) % R];
        if ((int)p <= p2) pl->pairs.push_back(make_int2((int)p, p2));
    }
    if (twr) stage_twiddles(pl->rp, *twr);
    if (twc) stage_twiddles(pl->cp, *twc);
    if (t4) {
        t4->resize((size_t)R * C);
        for (uint32_t p = 0; p < R; p++)
            for (uint32_t c = 0; c < C; c++)
                (*t4)[(size_t)p * C + c] = cis_neg((uint64_t)c * pl->rev_r[p] % H, H);
    }
    if (sw) {
        sw->resize((size_t)R * C);
        for (uint32_t p = 0; p < R; p++)
            for (uint32_t q = 0; q < C; q++)
                (*sw)[(size_t)p * C + q] =
                    cis_neg(((uint64_t)pl->rev_r[p] + (uint64_t)R * pl->rev_c[q]) % H, H);
    }
    if (part0) {
        part0->resize(C);
        for (uint32_t q = 0; q < C; q++) (*part0)[q] = pl->pos_c[(C - pl->rev_c[q]) % C];
    }
    if (part1) {
        part1->resize(C);
        for (uint32_t q = 0; q < C; q++) (*part1)[q] = pl->pos_c[C - 1 - pl->rev_c[q]];
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

std::shared_ptr<LengthPlan> get_plan(uint32_t L) {
    static std::mutex mu;
    static std::map<std::pair<int, uint32_t>, std::shared_ptr<LengthPlan>> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({dev, L});
    if (it != cache.end()) return it->second;
    std::vector<double2> twr, twc, t4, sw;
    std::vector<int> p0, p1;
    auto pl = build_plan_host(L, &twr, &twc, &t4, &sw, &p0, &p1);
    if (!pl) return nullptr;
    pl->device = dev;
    bool ok = upload(twr, &pl->twr, pl->device_bytes) && upload(twc, &pl->twc, pl->device_bytes) &&
              upload(t4, &pl->t4, pl->device_bytes) && upload(sw, &pl->sw, pl->device_bytes) &&
              upload(p0, &pl->part0, pl->device_bytes) && upload(p1, &pl->part1, pl->device_bytes) &&
              upload(pl->pairs, &pl->dpairs, pl->device_bytes);
    if (!ok) return nullptr;
    cache[{dev, L}] = pl;
    return pl;
}

}  // namespace kg
