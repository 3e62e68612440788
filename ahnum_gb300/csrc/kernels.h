// Host-side launch interface of the squaring kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "device.h"

namespace kg {

constexpr int kThreads = 256;
constexpr int kMinBlocks = 4;   // CTAs per SM the pass kernels are compiled for (64 registers)
constexpr int kMaxDevices = 64;  // devices tracked by the per-device tables of this library

// Control words of the persistent squaring kernel (device memory, zeroed before each launch):
// flow[kFlowNext] the next queue position, flow[kFlowTimeout] non-zero when a wait gave up,
// flow[kFlowDone + t] the items of test t finished in this launch.
constexpr int kFlowNext = 0;
constexpr int kFlowTimeout = 1;
constexpr int kFlowDone = 32;
// SM cycles a CTA of k_squarings waits for another CTA's item before it gives up (about 2 s)
constexpr long long kWaitCycles = 4000000000ll;

// Everything one launch of the pass kernels needs: the test table, the work lists and the
// grid sizes.  The same set serves a single test and a batch.
struct LaunchSet {
    cudaStream_t stream = nullptr;
    const TestDesc *tests = nullptr;   // device
    const WorkItem *rows = nullptr;    // device: row-pair work items
    int nrows = 0;
    const WorkItem *cols = nullptr;    // device: column-group work items
    int ncols = 0;
    const int *nrows_dev = nullptr;    // if set, the item counts are read on the device
    const int *ncols_dev = nullptr;    //   (graphs captured once, lists refilled per launch)
    int grid_rows = 0, grid_cols = 0;
    size_t row_smem_per_lane = 0;      // C * sizeof(double2) for the longest row
    size_t col_smem = 0;               // R * G * sizeof(double2) for the longest column
    int G = kGroup;                    // column-group width of every test in the launch
    int threads = kThreads;            // block size: 256, or 128 for twice the CTAs per SM
};

// Raise (never lower) the kernels' dynamic shared-memory limits on the current device; 0 on
// success.
int kernels_prepare(size_t row_smem, size_t col_smem);

// x, y non-null override the per-test operands (single-test use).  `step` is the index of
// this squaring within a launch sequence: tests whose count is <= step sit it out.
void launch_rows(const LaunchSet &s, bool mul, double2 *x, const double2 *y, int step = 0);
void launch_col_inverse(const LaunchSet &s, bool track_err, const double2 *x, int step = 0);
void launch_col_forward(const LaunchSet &s, double2 *x, bool use_slots, int step = 0);
// FP64 FMA throughput probe: `iters` dependent-chain DFMAs per thread over grid x block;
// the result is written to out[0] only if the chains overflow (never).
void launch_fp64_probe(cudaStream_t st, int grid, int block, int iters, double *out);
// The probe with `chains` chains per thread (4, 8 or 16 for DFMA; 8 for DMUL and DADD) of
// opcode op (0 DFMA, 1 DMUL, 2 DADD); -1 for a combination it does not have.
int launch_fp64_probe_var(cudaStream_t st, int grid, int block, int iters, int chains, int op, double *out);
// The digits of x (every test of the set's column list) into each test's dig scratch, or into
// `dig` when it is given (a single-test set).
void launch_col_digits(const LaunchSet &s, const double2 *x, long long *dig = nullptr);
// Zero test of a - b (mod N) for digit vectors of test `test` of the table (k_equal_mod_n, one
// CTA): *flag = 1 equal, 0 different, 2 undetermined (compare on the host).  a is overwritten.
void launch_equal(cudaStream_t st, const TestDesc *tests, int test, long long *a, const long long *b, int *flag);
// Squarings step0 .. step0+nsteps-1 of every test of the lists in one persistent launch
// (k_squarings) of `grid` CTAs.  `flow` holds kFlowDone + (tests) words, zeroed before the
// launch.  A CTA that waits longer than wait_limit SM cycles for another's item raises
// flow[kFlowTimeout] and the launch winds down.  Returns -1 if grid < 1.
int launch_squarings(const LaunchSet &s, unsigned *flow, int step0, int nsteps, int grid,
                     long long wait_limit = kWaitCycles);
// CTAs of k_squarings that fit at once on nsm SMs for this set (0 if none); call it outside
// stream capture.
int squarings_grid(const LaunchSet &s, int nsm);
size_t squarings_smem(size_t row_smem, size_t col_smem);
// op: 0 copy, 1 add, 2 sub
void launch_elementwise(cudaStream_t st, double2 *x, const double2 *y, size_t n, int op);

}  // namespace kg
