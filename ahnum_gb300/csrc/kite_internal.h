// Internal layout of the opaque kite_ctx / kite_num of this library.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "../../include/kite_ntt.h"
#include "layout.h"

struct kite_ctx {
    kg::Layout lay;            // exact digit layout, weights, N
    kc_engine *eng = nullptr;  // FP64 IBDWT engine for this modulus, or
    kn_engine *ntt = nullptr;  // the integer-NTT engine (KITE_BACKEND_CUDA_NTT)
    std::vector<int64_t> dig;  // L digits of host scratch
};

struct kite_num {
    void *d = nullptr;  // device memory: kc_num_doubles() doubles, or kn_num_words() words
};

// x <- x^2 + c, count times, on the context's engine (the LLR doubling with c = -2)
int kite_square_add_internal(kite_ctx *ctx, kite_num *x, uint64_t count, int64_t c);
// a == b (mod N): decided on the device by the FP64 engine (kc_equal: 4 bytes read back), by
// canonical limbs for the integer-NTT engine.  1 equal, 0 different, negative on a CUDA error.
int kite_equal_internal(kite_ctx *ctx, const kite_num *a, const kite_num *b);
