// Batched engine: many independent Fermat / LLR tests with different k, n and FFT lengths
// advanced together on one GPU (include/kite_cuda.h, kc_batch_*).
//
// The reference runs concurrent tests as independent contexts on CPU threads
// (tools/kite.c:65-105, `kite throughput`).  Here every test is a slot with its own modulus
// tables and numbers in device memory, and one launch of each pass kernel covers all slots: the
// work lists name (slot, row pair) and (slot, column group) items of every length.  A Gerbicz
// block of B squarings is one CUDA graph of 3*B kernel nodes, captured once; each replay reads
// the current slot table and work lists from device memory, and a slot that needs fewer than B
// squarings in a block (a tail) sits out the remaining steps.
//
// Each slot follows the reference's Fermat driver (src/prp.c:407-567): blocks of B squarings
// with d <- d*x at the end of each, a check d == x0 * t^(2^B) every M blocks (the check's
// squarings are batched like any other), rollback to the last verified state on a mismatch,
// restart at a longer FFT on round-off above 0.40, the tail computed twice.  LLR slots run the
// doubling V <- V^2 - 2 with the constant folded into the normaliser (src/llr.c:395-406).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "engine_internal.h"
#include "persist.h"

using namespace kg;

namespace {

enum class Phase { Free, Run, Check, TailX, TailT, Llr, Done, Failed };

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Slot {
    bool used = false;
    int kind = KC_TEST_FERMAT;
    uint64_t k = 0, n = 0;
    uint32_t base = 3;
    kc_engine *e = nullptr;
    double *x = nullptr, *d = nullptr, *x0 = nullptr, *t = nullptr, *vx = nullptr, *vd = nullptr;
    Phase phase = Phase::Free;
    uint64_t i = 0, vi = 0, full = 0, total = 0;
    uint32_t round_blocks = 0, consecutive_fail = 0, tail_attempts = 0;
    int count = 0;             // squarings this slot takes in the current block
    size_t bytes = 0;          // device bytes held
    int nadd = 0;              // LLR: digits of the constant -2
    int addj[kMaxAddend] = {};
    long long addv[kMaxAddend] = {};
    kc_test_result res{};
    double t_start = 0;
};

size_t slot_bytes(uint32_t L, uint32_t R, uint32_t NG) {
    // six numbers, two digit vectors, tables (bits, w, osc, idig), carry slots
    return (size_t)L * (6 * 8 + 2 * 8 + 1 + 3 * 8) + (size_t)NG * R * 8 + 4096;
}

}  // namespace

constexpr int kMaxParts = 4;  // most streams a split block uses

struct kc_batch {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    uint32_t B = 1000, M = 250;
    double maxround = 0.40;
    size_t budget = 0, in_use = 0;
    std::vector<Slot> slots;
    // device and pinned host mirrors of the work lists
    struct Lists {
        int cap_tests = 0, cap_rows = 0, cap_cols = 0;
        TestDesc *d_desc = nullptr, *h_desc = nullptr;
        WorkItem *d_rows = nullptr, *h_rows = nullptr, *d_cols = nullptr, *h_cols = nullptr;
        int *d_cnt = nullptr, *h_cnt = nullptr;
        unsigned *d_flow = nullptr;  // control words of the persistent kernel (kernels.h)
    } lists[2 + kMaxParts - 1];  // [0] squaring blocks (part 0 of a split block), [1] products,
                                 // [2 ..] parts 1 .. of a split block
    unsigned long long *h_err = nullptr;  // pinned, one per slot
    int cap_err = 0;
    int *d_eq = nullptr, *h_eq = nullptr;  // zero-test verdicts of the slots compared this block
    int cap_eq = 0;
    cudaGraphExec_t graph = nullptr;
    size_t graph_row_smem = 0, graph_col_smem = 0;
    uint32_t graph_B = 0;
    int grid = 0;
    int threads = 128;  // block size of the pass kernels
    bool persistent = false;      // squaring blocks as the persistent kernel k_squarings
    bool stagger = false;         // first rounds of 1..M blocks by admission order (kc_batch_stagger_checks)
    uint64_t admitted = 0;        // Fermat slots admitted so far
    int parts = 3;                // per-pass blocks of 2+ tests in this many parts, one stream each
    int form = -1;                // the form of the captured block graph (BlockForm)
    int graph_parts = 0;          // its number of parts
    cudaStream_t pstream[kMaxParts] = {};  // [0] is `stream`; [1 ..] the other parts of a split block
    cudaEvent_t fork = nullptr;            // split blocks: the other streams start after it
    cudaEvent_t join[kMaxParts] = {};      //   and `stream` waits for each of theirs
    uint32_t steps_per_launch = 100;
    unsigned *h_flow = nullptr;   // pinned: the timeout word read back after each block
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int err = 0;
    const char *what = "";      // the step that failed, for kc_batch_error_string
    uint64_t h2d = 0, d2h = 0;  // bytes moved by the current / last step
};

namespace {

bool bok(kc_batch *b, cudaError_t rc) {
    if (rc != cudaSuccess && !b->err) b->err = -(int)rc;
    return rc == cudaSuccess;
}

// a failure that is not a CUDA error: remember which step, return -1
int fail(kc_batch *b, const char *what) {
    b->what = what;
    return b->err ? b->err : -1;
}

void free_lists(kc_batch::Lists &l) {
    cudaFree(l.d_desc);
    cudaFree(l.d_rows);
    cudaFree(l.d_cols);
    cudaFree(l.d_cnt);
    cudaFree(l.d_flow);
    if (l.h_desc) cudaFreeHost(l.h_desc);
    if (l.h_rows) cudaFreeHost(l.h_rows);
    if (l.h_cols) cudaFreeHost(l.h_cols);
    if (l.h_cnt) cudaFreeHost(l.h_cnt);
    l = kc_batch::Lists{};
}

bool grow_lists(kc_batch *b, kc_batch::Lists &l, int tests, int rows, int cols) {
    if (tests <= l.cap_tests && rows <= l.cap_rows && cols <= l.cap_cols) return true;
    free_lists(l);
    l.cap_tests = std::max(tests, 64) * 2;
    l.cap_rows = std::max(rows, 1024) * 2;
    l.cap_cols = std::max(cols, 1024) * 2;
    return bok(b, cudaMalloc((void **)&l.d_desc, l.cap_tests * sizeof(TestDesc))) &&
           bok(b, cudaMalloc((void **)&l.d_rows, l.cap_rows * sizeof(WorkItem))) &&
           bok(b, cudaMalloc((void **)&l.d_cols, l.cap_cols * sizeof(WorkItem))) &&
           bok(b, cudaMalloc((void **)&l.d_cnt, 2 * sizeof(int))) &&
           bok(b, cudaMalloc((void **)&l.d_flow, (kFlowDone + l.cap_tests) * sizeof(unsigned))) &&
           bok(b, cudaMemsetAsync(l.d_flow, 0, (kFlowDone + l.cap_tests) * sizeof(unsigned), b->stream)) &&
           bok(b, cudaMallocHost((void **)&l.h_desc, l.cap_tests * sizeof(TestDesc))) &&
           bok(b, cudaMallocHost((void **)&l.h_rows, l.cap_rows * sizeof(WorkItem))) &&
           bok(b, cudaMallocHost((void **)&l.h_cols, l.cap_cols * sizeof(WorkItem))) &&
           bok(b, cudaMallocHost((void **)&l.h_cnt, 2 * sizeof(int)));
}

LaunchSet launch_set(kc_batch *b, const kc_batch::Lists &l, size_t row_lane, size_t col_smem) {
    LaunchSet s;
    s.stream = b->stream;
    s.tests = l.d_desc;
    s.rows = l.d_rows;
    s.cols = l.d_cols;
    s.nrows = l.cap_rows;
    s.ncols = l.cap_cols;
    s.nrows_dev = l.d_cnt;
    s.ncols_dev = l.d_cnt + 1;
    s.grid_rows = b->grid;
    s.grid_cols = b->grid;
    s.threads = b->threads;
    s.row_smem_per_lane = row_lane;
    s.col_smem = col_smem;
    return s;
}

void max_smem(kc_batch *b, size_t &row_lane, size_t &col) {
    row_lane = col = 0;
    for (auto &s : b->slots) {
        if (!s.used || !s.e) continue;
        row_lane = std::max(row_lane, s.e->ls.row_smem_per_lane);
        col = std::max(col, s.e->ls.col_smem);
    }
}

void release_numbers(Slot &s) {
    if (!s.e) return;
    for (double **p : {&s.x, &s.d, &s.x0, &s.t, &s.vx, &s.vd}) {
        if (*p) kc_num_free(s.e, *p);
        *p = nullptr;
    }
    kc_engine_free(s.e);
    s.e = nullptr;
}

void release_slot(kc_batch *b, Slot &s) {
    release_numbers(s);
    b->in_use -= std::min(b->in_use, s.bytes);
    s.bytes = 0;
}

bool alloc_numbers(Slot &s) {
    for (double **p : {&s.x, &s.d, &s.x0, &s.t, &s.vx, &s.vd}) {
        *p = kc_num_alloc(s.e);
        if (!*p) return false;
    }
    return true;
}

// x0 = base^k: exact while base^k < N, else square-and-multiply (src/prp.c:298-327)
bool power_start(Slot &s) {
    kc_engine *e = s.e;
    const size_t nl = e->lay.nlimbs;
    std::vector<uint64_t> l(nl, 0);
    l[0] = 1;
    if ((double)s.k * std::log2((double)s.base) + 2 < (double)s.n) {
        size_t used = 1;
        for (uint64_t i = 0; i < s.k; i++) {
            unsigned __int128 c = 0;
            for (size_t j = 0; j < used; j++) {
                c += (unsigned __int128)l[j] * s.base;
                l[j] = (uint64_t)c;
                c >>= 64;
            }
            if (c && used < nl) l[used++] = (uint64_t)c;
        }
        return kc_set_limbs(e, s.x0, l.data()) == 0;
    }
    if (kc_set_limbs(e, s.x0, l.data())) return false;
    for (int bit = 63; bit >= 0; bit--) {
        if (s.k >> bit == 0) continue;
        if (kc_square(e, s.x0, 1)) return false;
        if (((s.k >> bit) & 1) && kc_mul_small_host(e, s.x0, s.base)) return false;
    }
    return kc_sync(e) == 0;
}

bool open_engine(kc_batch *b, Slot &s, uint32_t L) {
    cudaSetDevice(b->device);
    s.e = kc_engine_create(s.k, s.n, L, nullptr, nullptr, nullptr, 0, 0, 0, 0, b->device, true);
    if (!s.e) return false;
    s.res.fft_len = L;
    return alloc_numbers(s);
}

// Fermat slot from verified limbs (or from x0 when vx is empty)
bool start_fermat(Slot &s, const std::vector<uint64_t> *vx, const std::vector<uint64_t> *vd) {
    kc_engine *e = s.e;
    if (!power_start(s)) return false;
    if (vx) {
        if (kc_set_limbs(e, s.x, vx->data()) || kc_set_limbs(e, s.d, vd->data())) return false;
    } else {
        if (kc_copy(e, s.x, s.x0) || kc_copy(e, s.d, s.x0)) return false;
    }
    if (kc_copy(e, s.vx, s.x) || kc_copy(e, s.vd, s.d)) return false;
    kc_reset_maxerr(e);
    s.i = s.vi;
    s.round_blocks = 0;
    s.phase = Phase::Run;
    return kc_sync(e) == 0;
}

// LLR slot: Lucas ladder for V_k(P, -1) on the slot's engine, then V_{2k} = V_k^2 + 2
// (src/llr.c:150-184, 395-401); the doublings that follow are batched.
bool start_llr(Slot &s, const std::vector<uint64_t> *vx) {
    kc_engine *e = s.e;
    std::vector<uint64_t> l(e->lay.nlimbs, 0);
    if (vx) {
        if (kc_set_limbs(e, s.x, vx->data())) return false;
    } else {
        double *v1 = s.d, *t = s.t, *cP = s.x0, *c2 = s.vd;  // borrowed until the ladder ends
        l[0] = s.res.P;
        if (kc_set_limbs(e, cP, l.data())) return false;
        l[0] = 2;
        if (kc_set_limbs(e, c2, l.data()) || kc_copy(e, s.x, c2) || kc_copy(e, v1, cP)) return false;
        uint64_t m = 0;
        int top = 63;
        while (top > 0 && !((s.k >> top) & 1)) top--;
        for (int bit = top; bit >= 0; bit--) {
            const bool odd = m & 1;
            kc_copy(e, t, s.x);
            kc_mul(e, t, v1);
            if (odd) kc_add(e, t, cP);
            else kc_sub(e, t, cP);
            if ((s.k >> bit) & 1) {
                kc_square(e, v1, 1);
                if (odd) kc_sub(e, v1, c2);
                else kc_add(e, v1, c2);
                kc_copy(e, s.x, t);
                m = 2 * m + 1;
            } else {
                kc_square(e, s.x, 1);
                if (odd) kc_add(e, s.x, c2);
                else kc_sub(e, s.x, c2);
                kc_copy(e, v1, t);
                m = 2 * m;
            }
        }
        if (kc_square_add(e, s.x, 1, 2)) return false;
        s.vi = 1;
    }
    uint32_t idx[kMaxAddend];
    int64_t val[kMaxAddend];
    s.nadd = e->lay.constant_digits(-2, idx, val, kMaxAddend);
    if (s.nadd < 0) return false;
    for (int j = 0; j < s.nadd; j++) {
        s.addj[j] = (int)idx[j];
        s.addv[j] = val[j];
    }
    if (kc_copy(e, s.vx, s.x)) return false;
    const double me = kc_maxerr(e);
    if (me > s.res.maxerr && me < 1.0) s.res.maxerr = me;
    kc_reset_maxerr(e);
    s.i = s.vi;
    s.total = s.n - 1;
    s.phase = s.i >= s.total ? Phase::Done : Phase::Llr;
    return kc_sync(e) == 0;
}

// The verdict of a comparison queued on the device this block (1 equal, 0 different); 2 (the
// device carry did not settle) falls back to canonical limbs on the host.
bool numbers_equal(Slot &s, const double *a, const double *c, int verdict) {
    if (verdict == 0 || verdict == 1) return verdict == 1;
    const size_t nl = s.e->lay.nlimbs;
    std::vector<uint64_t> la(nl), lc(nl);
    if (kc_get_limbs(s.e, a, la.data()) || kc_get_limbs(s.e, c, lc.data())) return false;
    return la == lc;
}

// the pair a slot compares after this block's products: d with x0 * t^(2^B) in its check, x
// with t after the doubled tail
bool compared_pair(Slot &s, const double *&a, const double *&c) {
    if (s.phase == Phase::Check) {
        a = s.t;
        c = s.d;
        return true;
    }
    if (s.phase == Phase::TailT) {
        a = s.x;
        c = s.t;
        return true;
    }
    return false;
}

void finish_fermat(Slot &s) {
    const size_t nl = s.e->lay.nlimbs;
    std::vector<uint64_t> y(nl);
    if (kc_get_limbs(s.e, s.x, y.data())) {
        s.res.rc = -1;
        s.phase = Phase::Failed;
        return;
    }
    bool prp = y[0] == (uint64_t)s.base * s.base;
    for (size_t j = 1; j < nl; j++) prp &= y[j] == 0;
    if (residue_nm1(y.data(), s.e->lay.Nl.data(), nl, s.base)) s.res.rc = -4;
    s.res.res64 = y[0];
    s.res.is_prp = prp;
    s.phase = Phase::Done;
}

void finish_llr(Slot &s) {
    const size_t nl = s.e->lay.nlimbs;
    std::vector<uint64_t> y(nl);
    if (kc_get_limbs(s.e, s.x, y.data())) {
        s.res.rc = -1;
        s.phase = Phase::Failed;
        return;
    }
    bool zero = true;
    for (uint64_t v : y) zero &= v == 0;
    s.res.res64 = y[0];
    s.res.is_prp = zero;
    s.phase = Phase::Done;
}

// round-off above the limit: restart the slot from its verified state at a longer FFT
void round_fail(kc_batch *b, Slot &s) {
    const size_t nl = s.e->lay.nlimbs;
    std::vector<uint64_t> lx(nl), ld(nl);
    bool ok = kc_get_limbs(s.e, s.vx, lx.data()) == 0;
    if (s.kind == KC_TEST_FERMAT) ok = ok && kc_get_limbs(s.e, s.vd, ld.data()) == 0;
    const uint32_t L = s.res.fft_len;
    release_numbers(s);
    s.res.roundoff_retries++;
    const uint32_t nL = next_fft_len(L + L / 25);
    ok = ok && nL && s.res.roundoff_retries < 8 && open_engine(b, s, nL);
    if (ok) ok = s.kind == KC_TEST_FERMAT ? start_fermat(s, &lx, &ld) : start_llr(s, &lx);
    if (!ok) {
        s.res.rc = -2;
        s.phase = Phase::Failed;
    }
}

bool active(const Slot &s) {
    return s.used && (s.phase == Phase::Run || s.phase == Phase::Check || s.phase == Phase::TailX ||
                      s.phase == Phase::TailT || s.phase == Phase::Llr);
}

double *square_target(Slot &s) {
    return (s.phase == Phase::Check || s.phase == Phase::TailT) ? s.t : s.x;
}

// fill a list set from (slot, x, y) triples; returns false on allocation failure
struct Entry {
    Slot *s;
    double *x;
    const double *y;
    int count;
    int err_every;
    bool addend;
};

bool fill_lists(kc_batch *b, kc_batch::Lists &l, const std::vector<Entry> &ents) {
    int rows = 0, cols = 0;
    for (auto &en : ents) {
        rows += (int)en.s->e->plan->pairs.size();
        cols += (int)en.s->e->NG;
    }
    if (!grow_lists(b, l, (int)ents.size(), rows, cols)) return false;
    std::vector<std::pair<int, WorkItem>> rv, cv;
    for (size_t t = 0; t < ents.size(); t++) {
        const Entry &en = ents[t];
        TestDesc d = en.s->e->desc;
        d.x = (double2 *)en.x;
        d.y = (const double2 *)en.y;
        d.count = en.count;
        d.err_every = en.err_every;
        d.nadd = en.addend ? en.s->nadd : 0;
        for (int j = 0; j < d.nadd; j++) {
            d.addj[j] = en.s->addj[j];
            d.addv[j] = en.s->addv[j];
        }
        l.h_desc[t] = d;
        const LengthPlan &P = *en.s->e->plan;
        for (size_t p = 0; p < P.pairs.size(); p++) rv.push_back({(int)P.C, WorkItem{(int)t, (int)p}});
        for (uint32_t g = 0; g < en.s->e->NG; g++) cv.push_back({(int)P.R, WorkItem{(int)t, (int)g}});
    }
    // longest items first, so the grid-stride walk ends with the short ones
    auto by_size = [](const std::pair<int, WorkItem> &a, const std::pair<int, WorkItem> &c) { return a.first > c.first; };
    std::stable_sort(rv.begin(), rv.end(), by_size);
    std::stable_sort(cv.begin(), cv.end(), by_size);
    for (size_t i = 0; i < rv.size(); i++) l.h_rows[i] = rv[i].second;
    for (size_t i = 0; i < cv.size(); i++) l.h_cols[i] = cv[i].second;
    l.h_cnt[0] = (int)rv.size();
    l.h_cnt[1] = (int)cv.size();
    b->h2d += ents.size() * sizeof(TestDesc) + (rv.size() + cv.size()) * sizeof(WorkItem) + 2 * sizeof(int);
    return bok(b, cudaMemcpyAsync(l.d_desc, l.h_desc, ents.size() * sizeof(TestDesc), cudaMemcpyHostToDevice, b->stream)) &&
           bok(b, cudaMemcpyAsync(l.d_rows, l.h_rows, rv.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, b->stream)) &&
           bok(b, cudaMemcpyAsync(l.d_cols, l.h_cols, cv.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, b->stream)) &&
           bok(b, cudaMemcpyAsync(l.d_cnt, l.h_cnt, 2 * sizeof(int), cudaMemcpyHostToDevice, b->stream));
}

// The forms a block's squarings take: one launch per pass over all slots; the persistent kernel
// over all slots; or one launch per pass over `parts` groups of slots of about equal work, each
// on its own stream (forked and joined inside the graph), so that the groups fill one another's
// launch tails and low-occupancy passes.  Measured on GB300, ms per squaring of the batch:
//
//   tests (workload)     persistent  per pass  2 parts  3 parts  4 parts
//   32 (benchmark's)       0.159      0.148     0.137    0.132    0.129
//   64                     0.262      0.287     0.231    0.230    0.230
//   256                    0.906      1.010     0.893    0.892    0.895
//   16 (served mix)        0.233      0.229     0.220    0.213    0.213
//   48                     0.541      0.495     0.429    0.422    0.421
//
// So a block of two or more slots is split in three parts (KITE_GB300_BATCH_SPLIT=P picks P, 1
// keeps one stream), and the persistent kernel runs only when KITE_GB300_BATCH_PERSISTENT=1
// asks for it.
enum BlockForm { kPerPass = 0, kPersistent = 1, kSplit = 2 };

kc_batch::Lists &part_lists(kc_batch *b, int p) { return p == 0 ? b->lists[0] : b->lists[1 + p]; }

// (re)capture the B-squaring graph when the lists, the shared-memory needs or the form changed
bool ensure_graph(kc_batch *b, size_t row_lane, size_t col_smem, bool lists_moved, int form, int parts) {
    if (b->graph && !lists_moved && b->graph_B == b->B && row_lane <= b->graph_row_smem &&
        col_smem <= b->graph_col_smem && form == b->form && parts == b->graph_parts)
        return true;
    const kc_batch::Lists &l = b->lists[0];
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    row_lane = std::max(row_lane, b->graph_row_smem);
    col_smem = std::max(col_smem, b->graph_col_smem);
    if (kernels_prepare(row_lane * 6, col_smem)) {
        b->what = "raising the kernels' shared-memory limit";
        return false;
    }
    LaunchSet s = launch_set(b, l, row_lane, col_smem);
    cudaGraph_t g;
    b->form = form;
    b->graph_parts = parts;
    const int sq_grid = form == kPersistent ? squarings_grid(s, b->nsm) : 0;
    if (!bok(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal))) return false;
    bool launched = true;
    if (form == kPersistent) {
        // persistent launches of steps_per_launch squarings each; the queue position and the
        // per-test counters start at zero in every launch, the timeout word is left alone
        const size_t done_bytes = (size_t)l.cap_tests * sizeof(unsigned);
        for (uint32_t j = 0; j < b->B && launched; j += b->steps_per_launch) {
            const uint32_t n = std::min(b->steps_per_launch, b->B - j);
            launched = bok(b, cudaMemsetAsync(l.d_flow + kFlowNext, 0, sizeof(unsigned), b->stream)) &&
                       bok(b, cudaMemsetAsync(l.d_flow + kFlowDone, 0, done_bytes, b->stream)) &&
                       launch_squarings(s, l.d_flow, (int)j, (int)n, sq_grid) == 0;
        }
    } else if (form == kSplit) {
        // part 0 on the batch stream, part p on pstream[p], forked and joined by events
        LaunchSet ps[kMaxParts];
        for (int p = 0; p < parts; p++) {
            ps[p] = launch_set(b, part_lists(b, p), row_lane, col_smem);
            ps[p].stream = b->pstream[p];
        }
        launched = bok(b, cudaEventRecord(b->fork, b->stream));
        for (int p = 1; p < parts && launched; p++) launched = bok(b, cudaStreamWaitEvent(b->pstream[p], b->fork, 0));
        for (uint32_t j = 0; j < b->B && launched; j++) {
            for (int p = 0; p < parts; p++) {
                launch_rows(ps[p], false, nullptr, nullptr, (int)j);
                launch_col_inverse(ps[p], true, nullptr, (int)j);
                launch_col_forward(ps[p], nullptr, true, (int)j);
            }
        }
        for (int p = 1; p < parts && launched; p++)
            launched = bok(b, cudaEventRecord(b->join[p], b->pstream[p])) &&
                       bok(b, cudaStreamWaitEvent(b->stream, b->join[p], 0));
    } else {
        for (uint32_t j = 0; j < b->B; j++) {
            launch_rows(s, false, nullptr, nullptr, (int)j);
            launch_col_inverse(s, true, nullptr, (int)j);
            launch_col_forward(s, nullptr, true, (int)j);
        }
    }
    if (!bok(b, cudaStreamEndCapture(b->stream, &g))) return false;
    if (!launched) {
        cudaGraphDestroy(g);
        b->what = "capturing the block's launches";
        return false;
    }
    bool ok = bok(b, cudaGraphInstantiate(&b->graph, g, 0));
    cudaGraphDestroy(g);
    b->graph_B = b->B;
    b->graph_row_smem = row_lane;
    b->graph_col_smem = col_smem;
    return ok;
}

}  // namespace

extern "C" {

kc_batch *kc_batch_new(int device, uint32_t gerbicz_block, uint32_t gerbicz_blocks, size_t mem_budget) {
    kc_batch *b = new (std::nothrow) kc_batch();
    if (!b) return nullptr;
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) {
        delete b;
        return nullptr;
    }
    b->device = device;
    cudaSetDevice(device);
    b->B = gerbicz_block ? gerbicz_block : 1000;
    b->M = gerbicz_blocks ? gerbicz_blocks : std::max(b->B / 4, 8u);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    b->budget = mem_budget ? mem_budget : fr / 10 * 8;
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, device);
    // Block size of the pass kernels: 128 threads, so that 8 CTAs share an SM with the register
    // budget (64 per thread) of 4 CTAs of 256.  Measured on GB300 over the 256-test workload:
    // 1.034 s per 1000-squaring block at 128 threads, 1.103 s at 256 and 1.103 s at 64.
    // KITE_GB300_BATCH_THREADS=256 selects the larger blocks.
    b->threads = 128;
    if (const char *t = getenv("KITE_GB300_BATCH_THREADS")) b->threads = atoi(t) == 256 ? 256 : 128;
    b->grid = b->nsm * (kThreads * kMinBlocks / b->threads);
    // A Gerbicz block's squarings run as pass launches in parts on several streams (BlockForm);
    // KITE_GB300_BATCH_PERSISTENT=1 runs them as persistent launches of k_squarings instead
    // (steps_per_launch squarings each).
    if (const char *t = getenv("KITE_GB300_BATCH_PERSISTENT")) b->persistent = atoi(t) != 0;
    // KITE_GB300_BATCH_SPLIT=P splits per-pass blocks into P parts (1 or 0: one stream)
    if (const char *t = getenv("KITE_GB300_BATCH_SPLIT")) b->parts = std::max(1, std::min(atoi(t), kMaxParts));
    if (const char *t = getenv("KITE_GB300_STEPS_PER_LAUNCH")) {
        const int v = atoi(t);
        if (v > 0) b->steps_per_launch = (uint32_t)std::min(v, 1000);  // queue index stays far below 2^32
    }
    if (!bok(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) || !bok(b, cudaEventCreate(&b->ev0)) ||
        !bok(b, cudaEventCreate(&b->ev1)) || !bok(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming))) {
        kc_batch_free(b);
        return nullptr;
    }
    b->pstream[0] = b->stream;
    for (int p = 1; p < kMaxParts; p++)
        if (!bok(b, cudaStreamCreateWithFlags(&b->pstream[p], cudaStreamNonBlocking)) ||
            !bok(b, cudaEventCreateWithFlags(&b->join[p], cudaEventDisableTiming))) {
            kc_batch_free(b);
            return nullptr;
        }
    return b;
}

void kc_batch_free(kc_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto &s : b->slots) release_slot(b, s);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int p = 1; p < kMaxParts; p++)
        if (b->pstream[p]) cudaStreamSynchronize(b->pstream[p]);
    for (auto &l : b->lists) free_lists(l);
    if (b->h_err) cudaFreeHost(b->h_err);
    cudaFree(b->d_eq);
    if (b->h_eq) cudaFreeHost(b->h_eq);
    if (b->h_flow) cudaFreeHost(b->h_flow);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    for (int p = 1; p < kMaxParts; p++) {
        if (b->pstream[p]) cudaStreamDestroy(b->pstream[p]);
        if (b->join[p]) cudaEventDestroy(b->join[p]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    delete b;
}

static int admit(kc_batch *b, int kind, uint64_t k, uint64_t n, uint32_t base, uint32_t fft_len) {
    if (!(k & 1) || k >= (1ull << 30) || n < 8) return -1;
    const uint32_t L = fft_len ? fft_len : choose_fft_len(k, n);
    uint32_t R = 0, C = 0;
    if (!L || !choose_shape(L / 2, R, C)) return -1;
    const size_t need = slot_bytes(L, R, C / kGroup);
    if (b->in_use + need > b->budget) return -2;
    size_t id = 0;
    while (id < b->slots.size() && b->slots[id].used) id++;
    if (id == b->slots.size()) b->slots.emplace_back();
    Slot &s = b->slots[id];
    s = Slot{};
    s.used = true;
    s.kind = kind;
    s.k = k;
    s.n = n;
    s.base = base;
    s.bytes = need;
    s.t_start = now_s();
    s.res.kind = kind;
    s.res.k = k;
    s.res.n = n;
    b->in_use += need;
    bool ok = true;
    if (kind == KC_TEST_LLR) {
        uint64_t factor = 0;
        uint32_t P = 0;
        ok = kite_llr_choose_P(k, n, &P, &factor) == 0;
        s.res.P = P;
        if (ok && factor) {  // a small factor: finished without any squaring
            s.res.factor = factor;
            s.phase = Phase::Done;
            return (int)id;
        }
    }
    ok = ok && open_engine(b, s, L);
    if (ok) ok = kind == KC_TEST_FERMAT ? start_fermat(s, nullptr, nullptr) : start_llr(s, nullptr);
    if (ok) s.full = s.n / b->B * b->B;
    // staggered checks: the first round of the j-th admitted Fermat slot is 1 + (j mod M) blocks,
    // so the slots' checks spread evenly over the blocks instead of falling on the same one
    if (ok && kind == KC_TEST_FERMAT && b->stagger) s.round_blocks = b->M - 1 - (uint32_t)(b->admitted % b->M);
    if (ok && kind == KC_TEST_FERMAT) b->admitted++;
    if (!ok) {
        release_slot(b, s);
        s.used = false;
        return -1;
    }
    return (int)id;
}

int kc_batch_add_fermat(kc_batch *b, uint64_t k, uint64_t n, uint32_t base, uint32_t fft_len) {
    return admit(b, KC_TEST_FERMAT, k, n, base ? base : 3, fft_len);
}

int kc_batch_add_llr(kc_batch *b, uint64_t k, uint64_t n, uint32_t fft_len) {
    return admit(b, KC_TEST_LLR, k, n, 0, fft_len);
}

void kc_batch_stagger_checks(kc_batch *b, int on) { b->stagger = on != 0; }

int kc_batch_active(const kc_batch *b) {
    int c = 0;
    for (auto &s : b->slots) c += active(s);
    return c;
}

size_t kc_batch_bytes_in_use(const kc_batch *b) { return b->in_use; }
size_t kc_batch_budget(const kc_batch *b) { return b->budget; }

int kc_batch_step(kc_batch *b, uint32_t blocks, double *gpu_ms) {
    cudaSetDevice(b->device);
    double ms_total = 0;
    b->h2d = b->d2h = 0;
    for (uint32_t blk = 0; blk < blocks && !b->err; blk++) {
        // ---- squarings: every active slot squares its current number up to B times
        std::vector<Entry> sq;
        for (auto &s : b->slots) {
            if (!active(s)) continue;
            int cnt = (int)b->B;
            if (s.phase == Phase::TailX || s.phase == Phase::TailT) cnt = (int)(s.n - s.full);
            if (s.phase == Phase::Llr) cnt = (int)std::min<uint64_t>(b->B, s.total - s.i);
            s.count = cnt;
            const bool llr = s.phase == Phase::Llr;
            sq.push_back({&s, square_target(s), nullptr, cnt, llr ? 1 : 4, llr});
        }
        if (sq.empty()) break;
        size_t row_lane, col_smem;
        max_smem(b, row_lane, col_smem);
        int form = b->persistent ? kPersistent : kPerPass;
        const int nparts = form == kPerPass ? std::min<int>(b->parts, (int)sq.size()) : 1;
        if (nparts >= 2) form = kSplit;
        // the lists: all slots in part 0, or a split block's parts of about equal work (row pairs
        // and column groups), largest slots first, each to the part with the least work so far
        std::vector<Entry> part[kMaxParts];
        if (form == kSplit) {
            std::vector<Entry> order = sq;
            auto work = [](const Entry &en) { return en.s->e->plan->pairs.size() + (size_t)en.s->e->NG; };
            std::stable_sort(order.begin(), order.end(), [&](const Entry &a, const Entry &c) { return work(a) > work(c); });
            size_t load[kMaxParts] = {};
            for (auto &en : order) {
                const int h = (int)(std::min_element(load, load + nparts) - load);
                part[h].push_back(en);
                load[h] += work(en);
            }
        } else {
            part[0] = sq;
        }
        bool moved = false;
        for (int p = 0; p < nparts || p == 0; p++) {
            kc_batch::Lists &l = part_lists(b, p);
            const int cap_before = l.cap_tests + l.cap_rows + l.cap_cols;
            TestDesc *before = l.d_desc;
            if (!fill_lists(b, l, part[p])) return fail(b, "filling the squaring work lists");
            moved = moved || before != l.d_desc || cap_before != l.cap_tests + l.cap_rows + l.cap_cols;
        }
        if (!ensure_graph(b, row_lane, col_smem, moved, form, std::max(nparts, 1)))
            return fail(b, *b->what ? b->what : "capturing the block graph");
        bok(b, cudaEventRecord(b->ev0, b->stream));
        bok(b, cudaGraphLaunch(b->graph, b->stream));
        // ---- end of block products: d <- d*x (after t <- d) for running Fermat slots,
        //      t <- t*x0 for slots being checked
        std::vector<Entry> mu;
        for (auto &s : b->slots) {
            if (!s.used) continue;
            if (s.phase == Phase::Run) {
                bok(b, cudaMemcpyAsync(s.t, s.d, (size_t)s.e->lay.L * 8, cudaMemcpyDeviceToDevice, b->stream));
                mu.push_back({&s, s.d, s.x, 1, 1, false});
            } else if (s.phase == Phase::Check) {
                mu.push_back({&s, s.t, s.x0, 1, 1, false});
            }
        }
        if (!mu.empty()) {
            if (!fill_lists(b, b->lists[1], mu)) return fail(b, "filling the product work lists");
            LaunchSet ms = launch_set(b, b->lists[1], b->graph_row_smem, b->graph_col_smem);
            launch_rows(ms, true, nullptr, nullptr, 0);
            launch_col_inverse(ms, true, nullptr, 0);
            launch_col_forward(ms, nullptr, true, 0);
            bok(b, cudaGetLastError());
        }
        // ---- comparisons on the device: the check's d == x0 * t^(2^B) and the tail's x == t,
        //      one verdict word per slot read back with the round-off
        if ((int)b->slots.size() > b->cap_eq) {
            cudaFree(b->d_eq);
            if (b->h_eq) cudaFreeHost(b->h_eq);
            b->d_eq = b->h_eq = nullptr;
            b->cap_eq = (int)b->slots.size() * 2 + 16;
            if (!bok(b, cudaMalloc((void **)&b->d_eq, b->cap_eq * sizeof(int))) ||
                !bok(b, cudaMallocHost((void **)&b->h_eq, b->cap_eq * sizeof(int))))
                return b->err;
        }
        for (size_t i = 0; i < b->slots.size(); i++) {
            Slot &s = b->slots[i];
            const double *a, *c;
            if (!active(s) || !compared_pair(s, a, c)) continue;
            kc_queue_equal(s.e, b->stream, a, c, b->d_eq + i);
            bok(b, cudaGetLastError());
            bok(b, cudaMemcpyAsync(&b->h_eq[i], b->d_eq + i, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
            b->d2h += sizeof(int);
        }
        bok(b, cudaEventRecord(b->ev1, b->stream));
        // ---- round-off of every slot of this block
        if ((int)b->slots.size() > b->cap_err) {
            if (b->h_err) cudaFreeHost(b->h_err);
            b->cap_err = (int)b->slots.size() * 2 + 16;
            if (!bok(b, cudaMallocHost((void **)&b->h_err, b->cap_err * sizeof(unsigned long long)))) return b->err;
        }
        for (size_t i = 0; i < b->slots.size(); i++) {
            Slot &s = b->slots[i];
            if (!active(s)) continue;
            bok(b, cudaMemcpyAsync(&b->h_err[i], s.e->d_maxerr, 8, cudaMemcpyDeviceToHost, b->stream));
            b->d2h += 8;
            bok(b, cudaMemsetAsync(s.e->d_maxerr, 0, 8, b->stream));
        }
        if (b->form == kPersistent) {
            if (!b->h_flow && !bok(b, cudaMallocHost((void **)&b->h_flow, sizeof(unsigned)))) return b->err;
            bok(b, cudaMemcpyAsync(b->h_flow, b->lists[0].d_flow + kFlowTimeout, sizeof(unsigned),
                                   cudaMemcpyDeviceToHost, b->stream));
            b->d2h += sizeof(unsigned);
        }
        if (!bok(b, cudaStreamSynchronize(b->stream))) return b->err;
        if (b->form == kPersistent && *b->h_flow) {
            // a CTA gave up waiting for another's item: the block's numbers are not to be trusted
            b->err = -(int)cudaErrorLaunchTimeout;
            return fail(b, "a CTA of the persistent squaring kernel timed out waiting for another's item");
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        ms_total += ms;
        // ---- host state machines
        for (size_t i = 0; i < b->slots.size(); i++) {
            Slot &s = b->slots[i];
            if (!active(s)) continue;
            double e;
            std::memcpy(&e, &b->h_err[i], 8);
            if (e > s.res.maxerr) s.res.maxerr = e;
            s.res.squarings += (uint64_t)s.count + (s.phase == Phase::Run || s.phase == Phase::Check);
            if (e > b->maxround) {
                round_fail(b, s);
                continue;
            }
            switch (s.phase) {
            case Phase::Run:
                s.i += b->B;
                s.round_blocks++;
                if (s.round_blocks >= b->M || s.i >= s.full) s.phase = Phase::Check;
                break;
            case Phase::Check:
                if (numbers_equal(s, s.t, s.d, b->h_eq[i])) {
                    s.consecutive_fail = 0;
                    s.vi = s.i;
                    kc_copy(s.e, s.vx, s.x);
                    kc_copy(s.e, s.vd, s.d);
                    s.round_blocks = 0;
                    if (s.vi >= s.full) {
                        s.tail_attempts = 0;
                        kc_copy(s.e, s.t, s.x);
                        s.phase = s.n > s.full ? Phase::TailX : Phase::Done;
                        if (s.phase == Phase::Done) finish_fermat(s);
                    } else {
                        s.phase = Phase::Run;
                    }
                } else {
                    s.res.gerbicz_errors++;
                    if (++s.consecutive_fail > 5) {
                        s.res.rc = -3;
                        s.phase = Phase::Failed;
                        break;
                    }
                    kc_copy(s.e, s.x, s.vx);
                    kc_copy(s.e, s.d, s.vd);
                    s.i = s.vi;
                    s.round_blocks = 0;
                    s.phase = Phase::Run;
                }
                kc_sync(s.e);
                break;
            case Phase::TailX:
                s.phase = Phase::TailT;
                break;
            case Phase::TailT:
                if (numbers_equal(s, s.x, s.t, b->h_eq[i])) {
                    finish_fermat(s);
                } else if (++s.tail_attempts > 5) {
                    s.res.rc = -3;
                    s.phase = Phase::Failed;
                } else {
                    s.res.gerbicz_errors++;
                    kc_copy(s.e, s.x, s.vx);
                    kc_copy(s.e, s.t, s.vx);
                    kc_sync(s.e);
                    s.phase = Phase::TailX;
                }
                break;
            case Phase::Llr:
                s.i += (uint64_t)s.count;
                kc_copy(s.e, s.vx, s.x);
                s.vi = s.i;
                if (s.i >= s.total) finish_llr(s);
                kc_sync(s.e);
                break;
            default:
                break;
            }
            if (s.phase == Phase::Done || s.phase == Phase::Failed) s.res.seconds = now_s() - s.t_start;
        }
    }
    if (gpu_ms) *gpu_ms = ms_total;
    return b->err ? b->err : kc_batch_active(b);
}

int kc_batch_result(const kc_batch *b, int slot, kc_test_result *out) {
    if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) return -1;
    const Slot &s = b->slots[slot];
    if (out) {
        *out = s.res;
        out->iter = s.vi;
        out->position = s.phase == Phase::Done ? s.n : s.i;
        out->fft_len = s.res.fft_len;
    }
    if (s.phase == Phase::Done) return 1;
    if (s.phase == Phase::Failed) return 2;
    return 0;
}

int kc_batch_read(kc_batch *b, int slot, uint64_t *limbs) {
    if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used || !b->slots[slot].e) return -1;
    cudaSetDevice(b->device);
    if (!bok(b, cudaStreamSynchronize(b->stream))) return b->err;
    Slot &s = b->slots[slot];
    return kc_get_limbs(s.e, s.x, limbs);
}

int kc_batch_checkpoint(kc_batch *b, int slot, const char *path) {
    if (!path || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used || !b->slots[slot].e) return -1;
    cudaSetDevice(b->device);
    if (!bok(b, cudaStreamSynchronize(b->stream))) return -1;
    Slot &s = b->slots[slot];
    const size_t nl = s.e->lay.nlimbs;
    std::vector<uint64_t> vx(nl), vd(nl);
    if (kc_get_limbs(s.e, s.vx, vx.data())) return -1;
    if (s.kind == KC_TEST_FERMAT) {
        if (kc_get_limbs(s.e, s.vd, vd.data())) return -1;
        return prp_checkpoint_write(path, s.k, s.n, s.base, s.vi, s.res.fft_len, vx, vd) ? 0 : -1;
    }
    LlrCheckpointHeader h{};
    h.k = s.k;
    h.n = s.n;
    h.P = s.res.P;
    h.iter = s.vi;
    h.fft_len = s.res.fft_len;
    h.run = 0;
    return llr_checkpoint_write(path, h, vx) ? 0 : -1;
}

int kc_batch_debug_corrupt(kc_batch *b, int slot) {
    if (slot < 0 || slot >= (int)b->slots.size() || !active(b->slots[slot])) return -1;
    cudaSetDevice(b->device);
    if (!bok(b, cudaStreamSynchronize(b->stream))) return b->err;
    Slot &s = b->slots[slot];
    const uint32_t L = s.e->lay.L;
    std::vector<int64_t> d(L);
    if (kc_to_digits(s.e, s.x, d.data())) return -1;
    d[L / 3] += 1;
    if (kc_from_digits(s.e, s.x, d.data())) return -1;
    return kc_sync(s.e) ? -1 : 0;
}

void kc_batch_last_transfer(const kc_batch *b, uint64_t *h2d, uint64_t *d2h) {
    if (h2d) *h2d = b->h2d;
    if (d2h) *d2h = b->d2h;
}

void kc_batch_release(kc_batch *b, int slot) {
    if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used) return;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    release_slot(b, b->slots[slot]);
    b->slots[slot].used = false;
    b->slots[slot].phase = Phase::Free;
}

int kc_batch_error(const kc_batch *b) { return b->err; }

const char *kc_batch_error_string(const kc_batch *b) {
    if (b->err) return cudaGetErrorString((cudaError_t)(-b->err));
    return b->what;
}

int kc_batch_profile(kc_batch *b, uint32_t squarings, double *ms, double *flops) {
    cudaSetDevice(b->device);
    std::vector<Entry> sq;
    double fl[3] = {0, 0, 0};
    for (auto &s : b->slots) {
        if (!s.used || s.phase != Phase::Run) continue;
        bok(b, cudaMemcpyAsync(s.t, s.x, (size_t)s.e->lay.L * 8, cudaMemcpyDeviceToDevice, b->stream));
        sq.push_back({&s, s.t, nullptr, 1 << 30, 4, false});
        const LengthPlan &P = *s.e->plan;
        const double H = P.H, L = P.L;
        fl[0] += 10.0 * H * std::log2((double)P.C) + 10.0 * L;
        fl[1] += 5.0 * H * std::log2((double)P.R) + 7.0 * L;
        fl[2] += 5.0 * H * std::log2((double)P.R) + 7.0 * L;
    }
    if (sq.empty()) return -1;
    size_t row_lane, col_smem;
    max_smem(b, row_lane, col_smem);
    row_lane = std::max(row_lane, b->graph_row_smem);
    col_smem = std::max(col_smem, b->graph_col_smem);
    if (kernels_prepare(row_lane * 6, col_smem)) return -1;
    if (!fill_lists(b, b->lists[1], sq)) return b->err ? b->err : -1;
    LaunchSet s = launch_set(b, b->lists[1], row_lane, col_smem);
    cudaEvent_t ev[4];
    for (auto &e : ev) cudaEventCreate(&e);
    double acc[3] = {0, 0, 0};
    for (uint32_t j = 0; j < squarings; j++) {
        cudaEventRecord(ev[0], b->stream);
        launch_rows(s, false, nullptr, nullptr, (int)j);
        cudaEventRecord(ev[1], b->stream);
        launch_col_inverse(s, true, nullptr, (int)j);
        cudaEventRecord(ev[2], b->stream);
        launch_col_forward(s, nullptr, true, (int)j);
        cudaEventRecord(ev[3], b->stream);
        if (!bok(b, cudaEventSynchronize(ev[3]))) break;
        for (int q = 0; q < 3; q++) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
            acc[q] += t;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &sl : b->slots)
        if (sl.used && sl.phase == Phase::Run) kc_reset_maxerr(sl.e);
    for (int q = 0; q < 3; q++) {
        if (ms) ms[q] = acc[q] / (squarings ? squarings : 1);
        if (flops) flops[q] = fl[q];
    }
    return b->err;
}

int kc_batch_profile_steps(kc_batch *b, uint32_t squarings, double *ms, double *flops) {
    cudaSetDevice(b->device);
    if (squarings == 0) return -1;
    std::vector<Entry> sq;
    double fl = 0;
    for (auto &s : b->slots) {
        if (!s.used || s.phase != Phase::Run) continue;
        bok(b, cudaMemcpyAsync(s.t, s.x, (size_t)s.e->lay.L * 8, cudaMemcpyDeviceToDevice, b->stream));
        sq.push_back({&s, s.t, nullptr, 1 << 30, 4, false});
        const LengthPlan &P = *s.e->plan;
        const double H = P.H, L = P.L;
        fl += 10.0 * H * std::log2((double)P.C) + 10.0 * L + 2 * (5.0 * H * std::log2((double)P.R) + 7.0 * L);
    }
    if (sq.empty()) return -1;
    size_t row_lane, col_smem;
    max_smem(b, row_lane, col_smem);
    row_lane = std::max(row_lane, b->graph_row_smem);
    col_smem = std::max(col_smem, b->graph_col_smem);
    if (kernels_prepare(row_lane * 6, col_smem)) return -1;
    kc_batch::Lists &l = b->lists[1];
    if (!fill_lists(b, l, sq)) return b->err ? b->err : -1;
    LaunchSet s = launch_set(b, l, row_lane, col_smem);
    const size_t words = (size_t)kFlowDone + l.cap_tests;
    const int grid = squarings_grid(s, b->nsm);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float t = 0;
    int rc = 0;
    for (int rep = 0; rep < 2 && !rc; rep++) {  // the first launch warms up
        bok(b, cudaMemsetAsync(l.d_flow, 0, words * sizeof(unsigned), b->stream));
        cudaEventRecord(e0, b->stream);
        rc = launch_squarings(s, l.d_flow, 0, (int)squarings, grid);
        cudaEventRecord(e1, b->stream);
        if (!bok(b, cudaEventSynchronize(e1))) rc = b->err;
    }
    if (!rc) cudaEventElapsedTime(&t, e0, e1);
    unsigned timeout = 0;
    if (!rc && bok(b, cudaMemcpy(&timeout, l.d_flow + kFlowTimeout, sizeof timeout, cudaMemcpyDeviceToHost)) && timeout)
        rc = -1;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &sl : b->slots)
        if (sl.used && sl.phase == Phase::Run) kc_reset_maxerr(sl.e);
    if (ms) *ms = t;
    if (flops) *flops = fl * squarings;
    return rc ? rc : b->err;
}

double kc_fp64_probe_rate(int device, int blocks_per_sm, int threads, int chains, int op) {
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return -1;
    if (blocks_per_sm < 1 || blocks_per_sm > 32 || (threads != 128 && threads != 256)) return -1;
    cudaSetDevice(device);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return -1;
    cudaEvent_t a, c;
    cudaEventCreate(&a);
    cudaEventCreate(&c);
    double *out = nullptr;
    double best = -1;
    const int grid = nsm * blocks_per_sm, iters = 32768 / chains;
    if (cudaMalloc((void **)&out, sizeof(double)) == cudaSuccess &&
        launch_fp64_probe_var(st, grid, threads, iters, chains, op, out) == 0) {  // warm-up
        best = 0;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(a, st);
            launch_fp64_probe_var(st, grid, threads, iters, chains, op, out);
            cudaEventRecord(c, st);
            if (cudaEventSynchronize(c) != cudaSuccess) {
                best = -1;
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, a, c);
            const double lanes = (double)chains * iters * grid * threads;
            if (ms > 0) best = std::max(best, lanes / (ms * 1e-3));
        }
    }
    cudaFree(out);
    cudaEventDestroy(a);
    cudaEventDestroy(c);
    cudaStreamDestroy(st);
    return best;
}

double kc_fp64_peak(int device) {
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return 0;
    cudaSetDevice(device);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaStream_t st;
    cudaEvent_t a, c;
    double *out = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return 0;
    cudaEventCreate(&a);
    cudaEventCreate(&c);
    cudaMalloc((void **)&out, sizeof(double));
    const int grid = nsm * 4, block = 256, iters = 4096;
    launch_fp64_probe(st, grid, block, iters, out);  // warm-up
    double best = 0;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(a, st);
        launch_fp64_probe(st, grid, block, iters, out);
        cudaEventRecord(c, st);
        cudaEventSynchronize(c);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, c);
        const double flops = 2.0 * 8.0 * iters * (double)grid * block;
        if (ms > 0) best = std::max(best, flops / (ms * 1e-3));
    }
    cudaFree(out);
    cudaEventDestroy(a);
    cudaEventDestroy(c);
    cudaStreamDestroy(st);
    return best;
}

}  // extern "C"
