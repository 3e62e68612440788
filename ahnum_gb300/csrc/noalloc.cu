// kc_square_noalloc: one modular squaring that allocates no memory.
//
// Every other entry point of the engine keeps its digit and carry scratch in buffers that
// kc_engine_new allocated.  Some callers cannot allocate device memory at the time they need a
// squaring:
//   * plugins loaded into a host whose memory pool owns all of the device memory, so a
//     cudaMalloc of their own fails or evicts the host's data;
//   * latency-bound loops, where cudaMalloc/cudaFree synchronise the device and stall the
//     stream.
// This entry point serves them.  Its scratch (the integer digits between the two column
// kernels, the per-segment carries, and the slot table the kernels read) lives in one
// file-scope device array that every GPU which loads this library reserves until the process
// exits.  The caller still provides the engine (its read-only tables), the input and the output.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/kite_cuda.h"
#include "engine_internal.h"

using namespace kg;

namespace {

constexpr size_t kDescBytes = (sizeof(TestDesc) + 255) / 256 * 256;
constexpr size_t kDigBytes = (size_t)KC_NOALLOC_MAX_WORDS * sizeof(long long);
// one carry per (column group, row): at most H / 2 of them (groups of 2 columns)
constexpr size_t kSlotBytes = (size_t)KC_NOALLOC_MAX_WORDS / 2 / 2 * sizeof(long long);
constexpr size_t kScratchBytes = kDescBytes + kDigBytes + kSlotBytes;

}  // namespace

// The scratch itself: ~0.65 MB per device, shared by every call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Writes the call's test descriptor into the head of the scratch.  The descriptor travels as a
// kernel argument, which the launch copies when it is issued, so nothing of the caller's stack
// frame is read after the call returns and no host staging buffer is involved.
__global__ void k_noalloc_desc(TestDesc d, TestDesc *dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = d;
}

namespace {

std::mutex g_addr_mu;
unsigned char *g_addr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device with that device
// current.  The host-side symbol is only a stand-in: passing it to a kernel would fault.  The
// cached address belongs to the device's primary context: after a cudaDeviceReset the module
// is loaded again and this cache is stale, so a process that resets a device must not call
// kc_square_noalloc on it afterwards.
unsigned char *scratch_address(int device, int *err) {
    if (device < 0 || device >= kMaxDevices) {
        *err = KC_NOALLOC_BAD_ARGUMENT;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[device]) {
        void *p = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (rc != cudaSuccess) {
            *err = -(int)rc;
            return nullptr;
        }
        g_addr[device] = static_cast<unsigned char *>(p);
    }
    return g_addr[device];
}

}  // namespace

extern "C" int kc_square_noalloc(kc_engine *e, const double *x, double *y) {
    if (!e || !x || !y) return KC_NOALLOC_BAD_ARGUMENT;
    const LengthPlan &P = *e->plan;
    if (e->lay.L > KC_NOALLOC_MAX_WORDS || (size_t)e->NG * P.R * sizeof(long long) > kSlotBytes)
        return KC_NOALLOC_TOO_LARGE;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != e->device && cudaSetDevice(e->device) != cudaSuccess) return KC_NOALLOC_BAD_ARGUMENT;
    int rc = 0;
    unsigned char *base = scratch_address(e->device, &rc);
    if (base) {
        TestDesc d = e->desc;
        d.dig = reinterpret_cast<long long *>(base + kDescBytes);
        d.slot = reinterpret_cast<long long *>(base + kDescBytes + kDigBytes);
        d.nadd = 0;
        d.count = 1 << 30;
        d.err_every = 1;
        d.x = nullptr;
        d.y = nullptr;
        // Nothing here needs clearing between calls: the descriptor is rewritten by every call,
        // and the column inverse kernel writes every digit and every carry slot before the
        // column forward kernel reads them.
        cudaError_t c = cudaSuccess;
        if (x != y)
            c = cudaMemcpyAsync(y, x, (size_t)e->lay.L * sizeof(double), cudaMemcpyDeviceToDevice, e->stream);
        if (c == cudaSuccess) {
            k_noalloc_desc<<<1, 32, 0, e->stream>>>(d, reinterpret_cast<TestDesc *>(base));
            c = cudaGetLastError();
        }
        if (c == cudaSuccess) {
            LaunchSet s = e->ls;
            s.tests = reinterpret_cast<const TestDesc *>(base);
            launch_rows(s, false, reinterpret_cast<double2 *>(y), nullptr);
            launch_col_inverse(s, true, reinterpret_cast<const double2 *>(y));
            launch_col_forward(s, reinterpret_cast<double2 *>(y), true);
            c = cudaGetLastError();
        }
        if (c != cudaSuccess) {
            rc = -(int)c;
            kc_ok(e, c);
        }
    }
    if (prev >= 0 && prev != e->device) cudaSetDevice(prev);
    return rc;
}
