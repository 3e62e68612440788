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
    unsigned long long *d_maxerr = nullptr;
    int *d_status = nullptr;
    long long *h_dig = nullptr;      // pinned staging for digit transfers
    unsigned long long *h_err = nullptr;
    int err = 0;
    uint32_t err_every = 1;
    uint64_t op_count = 0;
    int add_cached = 0;              // constant currently folded in desc (0: none)
    int64_t add_c = 0;
};


// helpers shared with the batch engine (engine.cu)
bool kc_ok(kc_engine *e, cudaError_t rc);
int kc_get_limbs(kc_engine *e, const double *x, uint64_t *limbs);   // canonical, waits
int kc_set_limbs(kc_engine *e, double *x, const uint64_t *limbs);
int kc_mul_small_host(kc_engine *e, double *x, int64_t m);
