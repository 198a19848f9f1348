// kernels.h -- host-side launch interface of the two arithmetic modes.
#pragma once
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace posi {

// Device view of an ensemble; identical layout to POSI_NS::Dev.
struct DevView {
    int64_t n_sys, nmax, stride;
    double* bf;
    int64_t* bi;
    double* sf;
    int64_t* si;
    const double* roche;
    const double* tables;
    const int32_t* list;
    int32_t n_list;
    int32_t* step_flags;
    double* hist;
    double* rec;
    double* ias;
};

// OP_STEPS_REC: OP_STEPS writing the adjoint's step records to DevView::rec
// (FAST build only).
// OP_STEPS_SCHED: OP_STEPS under a balanced schedule (whfast_sched_kernel)
// OP_IAS15_STEPS: n_steps IAS15 steps (DevView::ias set)
enum KernelOp { OP_STEPS = 0, OP_INIT = 1, OP_GRAVITY = 2, OP_EFFECTS = 3, OP_STEPS_REC = 4, OP_STEPS_SCHED = 5,
                OP_IAS15_STEPS = 6 };

struct LaunchArgs {
    int op;
    int G;                 // lanes per system: 2, 4, 8, 16 or 32
    int64_t n_steps;       // OP_STEPS
    int ignore_terms;      // OP_GRAVITY
    double t_eval;         // OP_EFFECTS
    int evolution, dl, acc;
    // OP_STEPS_SCHED: blocks, and per warp slot (blocks * 8) the job and steps
    int sched_blocks;
    const int32_t* slot_job;
    const int32_t* slot_steps;
};

// Returns cudaSuccess or the launch error.
cudaError_t launch_exact(const DevView& d, const LaunchArgs& a, cudaStream_t stream);
cudaError_t launch_fast(const DevView& d, const LaunchArgs& a, cudaStream_t stream);
// Kernel attributes (dynamic shared memory); call before the first launch.
cudaError_t prepare_exact();
cudaError_t prepare_fast();
// The IAS15 kernels (their own translation units; launch_exact / launch_fast
// forward OP_IAS15_STEPS to them).
cudaError_t launch_ias15_exact(const DevView& d, const LaunchArgs& a, cudaStream_t stream);
cudaError_t launch_ias15_fast(const DevView& d, const LaunchArgs& a, cudaStream_t stream);
cudaError_t prepare_ias15_exact();
cudaError_t prepare_ias15_fast();

// Lanes per system used for a system of n bodies (0 when n is out of range).
inline int group_size_for(int64_t n) {
    if (n < 1) return 0;
    if (n <= 2) return 2;
    if (n <= 4) return 4;
    if (n <= 8) return 8;
    if (n <= 16) return 16;
    if (n <= 32) return 32;
    return 0;
}

constexpr int kBlockThreads = 128;
// the balanced schedule's blocks: one per SM, eight warps (two per SMSP)
constexpr int kSchedBlockThreads = 256;

// Adjoint kernels (adjoint.cu): which = 0 records a chunk's tape, 1 runs its
// reverse sweep.  Systems of up to 8 bodies, Jacobi coordinates.
struct AdjView {
    int64_t n_sys, nmax, stride;
    const double* bf;
    const int64_t* bi;
    const double* sf;
    const int64_t* si;
    const int32_t* list;
    int32_t n_list;
    double* tape;
    double* lam;
    double* grad;
    int32_t* err;
};
int adjoint_group_size(int64_t n);
constexpr int kAdjTapeFields = 27 + 2 * (1 + 9 * 10);  // per-step record of the adjoint, doubles per body
cudaError_t launch_adjoint(const AdjView& v, int which, int64_t k_steps, int G, cudaStream_t stream);
cudaError_t prepare_adjoint();

// Sets the message posi_last_error() returns on the calling thread.
void set_last_error(const std::string& msg);

}  // namespace posi
