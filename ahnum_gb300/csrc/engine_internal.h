// Internal state of a single-modulus engine, shared by engine.cu and the batch engine.
#pragma once

#include <cuda_runtime.h>

#include <memory>

#include "../../include/kite_cuda.h"
#include "device.h"
#include "kernels.h"
#include "layout.h"
#include "plan.h"

struct kc_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    kg::Layout lay;
    std::shared_ptr<kg::LengthPlan> plan;
    kg::TestDesc desc{};
    kg::TestDesc *d_desc = nullptr;
    kg::WorkItem *d_work = nullptr;  // rows then columns
    kg::LaunchSet ls;
    uint8_t *d_bits = nullptr;
    double *d_w = nullptr, *d_osc = nullptr, *d_idig = nullptr;
    long long *d_dig = nullptr, *d_slot = nullptr;
    long long *d_dig2 = nullptr;     // second digit vector of the zero test (kc_equal)
    int *d_eq = nullptr, *h_eq = nullptr;  // its verdict, on the device and pinned
    unsigned long long *d_maxerr = nullptr;
    int *d_status = nullptr;
    long long *h_dig = nullptr;      // pinned staging for digit transfers
    unsigned long long *h_err = nullptr;
    int err = 0;
    uint32_t err_every = 1;
    uint64_t op_count = 0;
    int add_cached = 0;              // constant currently folded in desc (0: none)
    int64_t add_c = 0;
    int G = 8;                       // columns per column group
    uint32_t NG = 0;                 // column groups, C / G
    // squarings of one number replayed from a CUDA graph (kSquareChunk of them per replay),
    // one graph per recently squared number
    struct SquareGraph {
        const double *x = nullptr;
        cudaGraphExec_t exec = nullptr;
        uint64_t last_use = 0;
    } graphs[4];
    uint64_t graph_clock = 0;
};

constexpr uint64_t kSquareChunk = 16;

// kc_engine_new for a test run alone (throughput = false: shape and group width chosen for the
// latency of one squaring) or for a batch slot (throughput = true: the throughput shape, G = 8).
kc_engine *kc_engine_create(uint64_t k, uint64_t n, uint32_t L, const uint8_t *bits, const double *w,
                            const double *oscale, uint32_t top_t, uint64_t top_st, uint32_t top_m,
                            uint64_t sL, int device, bool throughput);


// helpers shared with the batch engine (engine.cu)
bool kc_ok(kc_engine *e, cudaError_t rc);
int kc_get_limbs(kc_engine *e, const double *x, uint64_t *limbs);   // canonical, waits
int kc_set_limbs(kc_engine *e, double *x, const uint64_t *limbs);
int kc_mul_small_host(kc_engine *e, double *x, int64_t m);
// Queues the zero test of a - b (mod N) on `stream`: the digits of a into e->d_dig, of b into
// e->d_dig2, the verdict (1 equal, 0 different, 2 undetermined) into *flag.
void kc_queue_equal(kc_engine *e, cudaStream_t stream, const double *a, const double *b, int *flag);
