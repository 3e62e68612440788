// Internal layout of the opaque kite_ctx / kite_num of this library.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "layout.h"

struct kite_ctx {
    kg::Layout lay;            // exact digit layout, weights, N
    kc_engine *eng = nullptr;  // device engine for this modulus
    std::vector<int64_t> dig;  // L digits of host scratch
};

struct kite_num {
    double *d = nullptr;  // device memory, kc_num_doubles() doubles
};
