// Single-modulus engine behind the kc_* C ABI (include/kite_cuda.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/kite_cuda.h"
#include "kernels.h"
#include "layout.h"
#include "plan.h"
#include "engine_internal.h"

using namespace kg;

namespace {

}  // namespace

bool kc_ok(kc_engine *e, cudaError_t rc) {
    if (rc != cudaSuccess && !e->err) e->err = -(int)rc;
    return rc == cudaSuccess;
}

int kc_get_limbs(kc_engine *e, const double *x, uint64_t *limbs) {
    std::vector<int64_t> d(e->lay.L);
    if (kc_to_digits(e, x, d.data())) return e->err ? e->err : -1;
    e->lay.digits_to_limbs(d.data(), limbs);
    return 0;
}

int kc_set_limbs(kc_engine *e, double *x, const uint64_t *limbs) {
    std::vector<int64_t> d(e->lay.L);
    e->lay.limbs_to_digits(limbs, d.data());
    return kc_from_digits(e, x, d.data());
}

void kc_queue_equal(kc_engine *e, cudaStream_t stream, const double *a, const double *b, int *flag) {
    LaunchSet s = e->ls;
    s.stream = stream;
    launch_col_digits(s, (const double2 *)a, e->d_dig);
    launch_col_digits(s, (const double2 *)b, e->d_dig2);
    launch_equal(stream, e->d_desc, 0, e->d_dig, e->d_dig2, flag);
}

int kc_mul_small_host(kc_engine *e, double *x, int64_t m) {
    std::vector<int64_t> d(e->lay.L);
    if (kc_to_digits(e, x, d.data())) return e->err ? e->err : -1;
    for (auto &v : d) v *= m;
    e->lay.carry(d.data());
    return kc_from_digits(e, x, d.data());
}

namespace {

bool ok(kc_engine *e, cudaError_t rc) {
    if (rc != cudaSuccess && !e->err) e->err = -(int)rc;
    return rc == cudaSuccess;
}

bool check_launch(kc_engine *e) { return ok(e, cudaGetLastError()); }

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

template <class T>
bool dalloc(kc_engine *e, T **p, size_t count) {
    return ok(e, cudaMalloc((void **)p, (count ? count : 1) * sizeof(T)));
}

void release(kc_engine *e) {
    for (auto &g : e->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    cudaFree(e->d_desc);
    cudaFree(e->d_work);
    cudaFree(e->d_bits);
    cudaFree(e->d_w);
    cudaFree(e->d_osc);
    cudaFree(e->d_idig);
    cudaFree(e->d_dig);
    cudaFree(e->d_dig2);
    cudaFree(e->d_eq);
    if (e->h_eq) cudaFreeHost(e->h_eq);
    cudaFree(e->d_slot);
    cudaFree(e->d_maxerr);
    cudaFree(e->d_status);
    if (e->h_dig) cudaFreeHost(e->h_dig);
    if (e->h_err) cudaFreeHost(e->h_err);
    if (e->stream) cudaStreamDestroy(e->stream);
}

bool upload_desc(kc_engine *e) {
    return ok(e, cudaMemcpyAsync(e->d_desc, &e->desc, sizeof(TestDesc), cudaMemcpyHostToDevice, e->stream));
}

bool want_err(kc_engine *e) {
    bool t = e->err_every <= 1 || e->op_count % e->err_every == 0;
    e->op_count++;
    return t;
}

// one product pass: row pass (square or multiply), then the two column kernels
int product(kc_engine *e, double2 *x, const double2 *y) {
    const bool track = want_err(e);
    launch_rows(e->ls, y != nullptr, x, y);
    launch_col_inverse(e->ls, track, x);
    launch_col_forward(e->ls, x, true);
    return check_launch(e) ? 0 : e->err;
}

// A graph of kSquareChunk squarings of x (its kernels take x as an argument); the column
// inverse tracks round-off on the steps that are multiples of the descriptor's err_every.
cudaGraphExec_t square_graph(kc_engine *e, double2 *x) {
    kc_engine::SquareGraph *slot = nullptr;
    for (auto &g : e->graphs)
        if (g.exec && g.x == (const double *)x) slot = &g;
    if (!slot) {
        slot = &e->graphs[0];
        for (auto &g : e->graphs)
            if (!g.exec || g.last_use < slot->last_use) slot = &g;
        if (slot->exec) cudaGraphExecDestroy(slot->exec);
        slot->exec = nullptr;
        slot->x = (const double *)x;
        cudaGraph_t graph;
        if (!ok(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal))) return nullptr;
        for (uint64_t j = 0; j < kSquareChunk; j++) {
            launch_rows(e->ls, false, x, nullptr, (int)j);
            launch_col_inverse(e->ls, true, x, (int)j);
            launch_col_forward(e->ls, x, true, (int)j);
        }
        if (!ok(e, cudaStreamEndCapture(e->stream, &graph))) return nullptr;
        const bool inst = ok(e, cudaGraphInstantiate(&slot->exec, graph, 0));
        cudaGraphDestroy(graph);
        if (!inst) return nullptr;
    }
    slot->last_use = ++e->graph_clock;
    return slot->exec;
}

// count squarings of x: whole chunks from the graph, the rest launched one by one
int square_many(kc_engine *e, double2 *x, uint64_t count) {
    while (count >= kSquareChunk) {
        cudaGraphExec_t g = square_graph(e, x);
        if (!g || !ok(e, cudaGraphLaunch(g, e->stream))) return e->err ? e->err : -1;
        count -= kSquareChunk;
        e->op_count += kSquareChunk;
    }
    for (uint64_t i = 0; i < count; i++)
        if (product(e, x, nullptr)) return e->err;
    return 0;
}

int set_addend(kc_engine *e, int64_t c) {
    if (e->add_cached == (c != 0) && e->add_c == c) return 0;
    uint32_t idx[kMaxAddend];
    int64_t val[kMaxAddend];
    int cnt = 0;
    if (c) {
        cnt = e->lay.constant_digits(c, idx, val, kMaxAddend);
        if (cnt < 0) return -1;
    }
    e->desc.nadd = cnt;
    for (int i = 0; i < cnt; i++) {
        e->desc.addj[i] = (int)idx[i];
        e->desc.addv[i] = val[i];
    }
    e->add_cached = c != 0;
    e->add_c = c;
    return upload_desc(e) ? 0 : e->err;
}

}  // namespace

extern "C" {

kc_engine *kc_engine_new(uint64_t k, uint64_t n, uint32_t L, const uint8_t *bits, const double *w,
                         const double *oscale, uint32_t top_t, uint64_t top_st, uint32_t top_m,
                         uint64_t sL, int device) {
    return kc_engine_create(k, n, L, bits, w, oscale, top_t, top_st, top_m, sL, device, false);
}

}  // extern "C"

kc_engine *kc_engine_create(uint64_t k, uint64_t n, uint32_t L, const uint8_t *bits, const double *w,
                            const double *oscale, uint32_t top_t, uint64_t top_st, uint32_t top_m,
                            uint64_t sL, int device, bool throughput) {
    kc_engine *e = new (std::nothrow) kc_engine();
    if (!e) return nullptr;
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) {
        delete e;
        return nullptr;
    }
    e->device = device;
    DeviceGuard dg(device);
    if (!e->lay.build(k, n, L)) {
        delete e;
        return nullptr;
    }
    // a caller-provided layout must be the one this (k, n, L) defines
    if ((bits && std::memcmp(bits, e->lay.bits.data(), L)) || (top_t && top_t != e->lay.top_t) ||
        (top_st && top_st != e->lay.top_st) || (top_m && top_m != e->lay.top_m) || (sL && sL != e->lay.sL)) {
        delete e;
        return nullptr;
    }
    const double *wv = w ? w : e->lay.w.data();
    const double *ov = oscale ? oscale : e->lay.oscale.data();
    // a test run alone spreads each pass over the SMs (shape and column-group width chosen for
    // latency); a batch slot takes the throughput shape and the widest groups
    const unsigned top_digits = e->lay.L - e->lay.top_t;
    if (throughput) {
        e->G = kGroup;
        e->plan = get_plan(L);
    } else {
        unsigned min_bits = 64;
        for (uint8_t b : e->lay.bits) min_bits = b < min_bits ? b : min_bits;
        int nsm = 1;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
        uint32_t R = 0, C = 0;
        int G = kGroup;
        if (choose_latency_shape(L / 2, nsm, min_bits, top_digits, R, C, G)) {
            e->G = G;
            e->plan = get_plan(L, R);
        }
    }
    if (!e->plan || top_digits > 2 * (uint32_t)e->G) {
        delete e;
        return nullptr;
    }
    const LengthPlan &P = *e->plan;
    const uint32_t H = P.H;
    e->NG = P.C / e->G;
    bool good = ok(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) &&
                dalloc(e, &e->d_desc, 1) && dalloc(e, &e->d_work, P.pairs.size() + e->NG) &&
                dalloc(e, &e->d_bits, L) && dalloc(e, &e->d_w, L) && dalloc(e, &e->d_osc, L) &&
                dalloc(e, &e->d_idig, L) && dalloc(e, &e->d_dig, L) && dalloc(e, &e->d_dig2, L) &&
                dalloc(e, &e->d_eq, 1) && ok(e, cudaMallocHost((void **)&e->h_eq, sizeof(int))) &&
                dalloc(e, &e->d_slot, (size_t)e->NG * P.R) &&
                dalloc(e, &e->d_maxerr, 1) && dalloc(e, &e->d_status, 1) &&
                ok(e, cudaMallocHost((void **)&e->h_dig, (size_t)L * sizeof(long long))) &&
                ok(e, cudaMallocHost((void **)&e->h_err, sizeof(unsigned long long)));
    if (good) {
        std::vector<double> osc(L), idig(L);
        const double s4 = 1.0 / (4.0 * H);
        for (uint32_t j = 0; j < L; j++) {
            osc[j] = ov[j] * s4;
            idig[j] = 1.0 / ((double)P.R * wv[j]);
        }
        std::vector<WorkItem> work;
        for (size_t i = 0; i < P.pairs.size(); i++) work.push_back({0, (int)i});
        for (uint32_t g = 0; g < e->NG; g++) work.push_back({0, (int)g});
        good = ok(e, cudaMemcpy(e->d_bits, e->lay.bits.data(), L, cudaMemcpyHostToDevice)) &&
               ok(e, cudaMemcpy(e->d_w, wv, L * sizeof(double), cudaMemcpyHostToDevice)) &&
               ok(e, cudaMemcpy(e->d_osc, osc.data(), L * sizeof(double), cudaMemcpyHostToDevice)) &&
               ok(e, cudaMemcpy(e->d_idig, idig.data(), L * sizeof(double), cudaMemcpyHostToDevice)) &&
               ok(e, cudaMemcpy(e->d_work, work.data(), work.size() * sizeof(WorkItem), cudaMemcpyHostToDevice)) &&
               ok(e, cudaMemset(e->d_maxerr, 0, sizeof(unsigned long long))) &&
               ok(e, cudaMemset(e->d_status, 0, sizeof(int))) &&
               ok(e, cudaMemset(e->d_slot, 0, (size_t)e->NG * P.R * sizeof(long long)));
    }
    if (good) {
        TestDesc &d = e->desc;
        d.L = (int)L;
        d.H = (int)H;
        d.R = (int)P.R;
        d.C = (int)P.C;
        d.NG = (int)e->NG;
        d.G = e->G;
        d.rp = P.rp;
        d.cp = P.cp;
        d.twr = P.twr;
        d.twc = P.twc;
        d.t4 = P.t4;
        d.sw = P.sw;
        d.posr = P.dposr;
        d.posc = P.dposc;
        d.pairs = P.dpairs;
        d.npairs = (int)P.pairs.size();
        d.bits = e->d_bits;
        d.w = e->d_w;
        d.osc = e->d_osc;
        d.idig = e->d_idig;
        d.dig = e->d_dig;
        d.slot = e->d_slot;
        d.maxerr = e->d_maxerr;
        d.status = e->d_status;
        d.k = k;
        d.top_t = (int)e->lay.top_t;
        d.top_m = (int)e->lay.top_m;
        d.top_shift = (int)(e->lay.sL - e->lay.top_st);
        d.nadd = 0;
        d.x = nullptr;
        d.y = nullptr;
        d.count = 1 << 30;
        d.err_every = 1;
        good = upload_desc(e) && ok(e, cudaStreamSynchronize(e->stream));
        LaunchSet &s = e->ls;
        s.stream = e->stream;
        s.tests = e->d_desc;
        s.rows = e->d_work;
        s.nrows = (int)P.pairs.size();
        s.cols = e->d_work + P.pairs.size();
        s.ncols = (int)e->NG;
        s.grid_rows = s.nrows;
        s.grid_cols = s.ncols;
        s.row_smem_per_lane = (size_t)P.C * sizeof(double2);
        s.col_smem = (size_t)P.R * e->G * sizeof(double2);
        s.G = e->G;
        good = good && kernels_prepare(s.row_smem_per_lane * 6, s.col_smem) == 0;
    }
    if (!good) {
        release(e);
        delete e;
        return nullptr;
    }
    return e;
}

extern "C" {

void kc_engine_free(kc_engine *e) {
    if (!e) return;
    DeviceGuard dg(e->device);
    cudaStreamSynchronize(e->stream);
    release(e);
    delete e;
}

size_t kc_num_doubles(const kc_engine *e) { return e->lay.L; }

double *kc_num_alloc(kc_engine *e) {
    DeviceGuard dg(e->device);
    double *p = nullptr;
    if (!ok(e, cudaMalloc((void **)&p, (size_t)e->lay.L * sizeof(double)))) return nullptr;
    if (!ok(e, cudaMemsetAsync(p, 0, (size_t)e->lay.L * sizeof(double), e->stream))) {
        cudaFree(p);
        return nullptr;
    }
    return p;
}

void kc_num_free(kc_engine *e, double *x) {
    if (!x) return;
    DeviceGuard dg(e->device);
    cudaStreamSynchronize(e->stream);
    cudaFree(x);
}

int kc_from_digits(kc_engine *e, double *x, const int64_t *digits) {
    DeviceGuard dg(e->device);
    const size_t L = e->lay.L;
    if (!ok(e, cudaStreamSynchronize(e->stream))) return e->err;  // staging buffer reuse
    std::memcpy(e->h_dig, digits, L * sizeof(long long));
    if (!ok(e, cudaMemcpyAsync(e->d_dig, e->h_dig, L * sizeof(long long), cudaMemcpyHostToDevice, e->stream)))
        return e->err;
    launch_col_forward(e->ls, (double2 *)x, false);
    return check_launch(e) ? 0 : e->err;
}

int kc_to_digits(kc_engine *e, const double *x, int64_t *digits) {
    DeviceGuard dg(e->device);
    const size_t L = e->lay.L;
    launch_col_digits(e->ls, (const double2 *)x);
    if (!check_launch(e)) return e->err;
    if (!ok(e, cudaMemcpyAsync(e->h_dig, e->d_dig, L * sizeof(long long), cudaMemcpyDeviceToHost, e->stream)) ||
        !ok(e, cudaStreamSynchronize(e->stream)))
        return e->err;
    std::memcpy(digits, e->h_dig, L * sizeof(long long));
    return 0;
}

int kc_equal(kc_engine *e, const double *a, const double *b) {
    DeviceGuard dg(e->device);
    if (a == b) return 1;
    kc_queue_equal(e, e->stream, a, b, e->d_eq);
    if (!check_launch(e) ||
        !ok(e, cudaMemcpyAsync(e->h_eq, e->d_eq, sizeof(int), cudaMemcpyDeviceToHost, e->stream)) ||
        !ok(e, cudaStreamSynchronize(e->stream)))
        return e->err;
    if (*e->h_eq != 2) return *e->h_eq;
    // the device carry did not settle within its bounds: compare canonical limbs on the host
    std::vector<uint64_t> la(e->lay.nlimbs), lb(e->lay.nlimbs);
    if (kc_get_limbs(e, a, la.data()) || kc_get_limbs(e, b, lb.data())) return e->err ? e->err : -1;
    return la == lb ? 1 : 0;
}

int kc_square(kc_engine *e, double *x, uint64_t count) {
    DeviceGuard dg(e->device);
    if (e->add_c && set_addend(e, 0)) return e->err ? e->err : -1;
    return square_many(e, (double2 *)x, count);
}

int kc_square_add(kc_engine *e, double *x, uint64_t count, int64_t c) {
    DeviceGuard dg(e->device);
    if (set_addend(e, c)) return e->err ? e->err : -1;
    return square_many(e, (double2 *)x, count);
}

int kc_mul(kc_engine *e, double *x, const double *y) {
    DeviceGuard dg(e->device);
    if (e->add_c && set_addend(e, 0)) return e->err ? e->err : -1;
    return product(e, (double2 *)x, (const double2 *)y);
}

int kc_copy(kc_engine *e, double *dst, const double *src) {
    DeviceGuard dg(e->device);
    if (dst == src) return 0;
    return ok(e, cudaMemcpyAsync(dst, src, (size_t)e->lay.L * sizeof(double), cudaMemcpyDeviceToDevice, e->stream))
               ? 0
               : e->err;
}

int kc_add(kc_engine *e, double *x, const double *y) {
    DeviceGuard dg(e->device);
    launch_elementwise(e->stream, (double2 *)x, (const double2 *)y, e->lay.L / 2, 1);
    return check_launch(e) ? 0 : e->err;
}

int kc_sub(kc_engine *e, double *x, const double *y) {
    DeviceGuard dg(e->device);
    launch_elementwise(e->stream, (double2 *)x, (const double2 *)y, e->lay.L / 2, 2);
    return check_launch(e) ? 0 : e->err;
}

double kc_maxerr(kc_engine *e) {
    DeviceGuard dg(e->device);
    if (e->err) return 1.0;
    if (!ok(e, cudaMemcpyAsync(e->h_err, e->d_maxerr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, e->stream)) ||
        !ok(e, cudaStreamSynchronize(e->stream)))
        return 1.0;
    double v;
    std::memcpy(&v, e->h_err, sizeof v);
    return v;
}

void kc_reset_maxerr(kc_engine *e) {
    DeviceGuard dg(e->device);
    ok(e, cudaMemsetAsync(e->d_maxerr, 0, sizeof(unsigned long long), e->stream));
}

void kc_set_roundoff_check(kc_engine *e, uint32_t every) {
    e->err_every = every ? every : 1;
    if (e->desc.err_every != (int)e->err_every) {
        DeviceGuard dg(e->device);
        e->desc.err_every = (int)e->err_every;  // read by the graphed squarings
        upload_desc(e);
    }
}

int kc_error(const kc_engine *e) { return e->err; }

int kc_sync(kc_engine *e) {
    DeviceGuard dg(e->device);
    ok(e, cudaStreamSynchronize(e->stream));
    return e->err;
}

void *kc_stream(kc_engine *e) { return (void *)e->stream; }

void kc_shape(const kc_engine *e, uint32_t *R, uint32_t *C) {
    if (R) *R = e->plan->R;
    if (C) *C = e->plan->C;
}

int kc_group_width(const kc_engine *e) { return e->G; }

int kc_engine_wait_selftest(kc_engine *e, uint64_t wait_cycles) {
    DeviceGuard dg(e->device);
    int nsm = 0;
    if (!ok(e, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, e->device))) return e->err;
    // the engine's column items without its row items: every column item waits for row items
    // that are not in the queue, so every wait runs out
    LaunchSet s = e->ls;
    s.nrows = 0;
    s.nrows_dev = nullptr;
    s.ncols_dev = nullptr;
    const int grid = squarings_grid(s, nsm);
    const size_t bytes = (kFlowDone + 1) * sizeof(unsigned);
    unsigned *flow = nullptr;
    if (!ok(e, cudaMalloc((void **)&flow, bytes))) return e->err;
    int rc = -1;
    unsigned timed_out = 0;
    if (ok(e, cudaMemsetAsync(flow, 0, bytes, e->stream)) &&
        launch_squarings(s, flow, 0, 1, grid, (long long)wait_cycles) == 0 && check_launch(e) &&
        ok(e, cudaMemcpyAsync(&timed_out, flow + kFlowTimeout, sizeof timed_out, cudaMemcpyDeviceToHost, e->stream)) &&
        ok(e, cudaStreamSynchronize(e->stream)))
        rc = timed_out ? 1 : 0;
    else if (e->err)
        rc = e->err;
    cudaStreamSynchronize(e->stream);
    cudaFree(flow);
    return rc;
}

}  // extern "C"
