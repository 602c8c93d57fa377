// noalloc.cu -- nmg_rk4_step_noalloc: one RK4 step that allocates nothing.
//
// Who needs it: callers that cannot call cudaMalloc while they step, e.g. a
// host code whose device memory all comes from its own pool or from a
// framework allocator, code running where new device allocations are not
// allowed (inside a region that must not grow the memory footprint, or
// under an allocator that forbids raw cudaMalloc), or a solver that must
// not fail for lack of memory in the middle of a run.  They pass u in and u
// out; the two RK4 stage buffers come from one file-scope __device__ array
// of fixed size that every GPU loading this library holds until the
// process exits.
//
// Rules of use:
//  - At most NMG_NOALLOC_MAX_STATE doubles per state (2 stage buffers of
//    that size, 2 x 16 MiB); larger states are rejected with NMG_EINVAL.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture.
//  - All calls in the process share the one array: calls that overlap on
//    the GPU (from two contexts, streams or threads at the same time) race
//    on it and give wrong results.  Calls on one context are stream-ordered
//    and this function waits for its step to finish before returning.
//  - Nothing in the array has to start at zero: every stage writes a stage
//    buffer completely before the next stage reads it, and the stale
//    contents left by the previous call are never read.
//  - If the context has not been tuned yet, the step uses the first
//    compiled kernel variant instead of running the autotuner (which would
//    create CUDA events).
//  - The step is the one nmg_rk4_step takes: a context's MRS limiter and
//    exponential filter, if switched on, are applied where that entry point
//    applies them (their buffers were allocated when they were switched on).
//  - The context's device must be the current device; a call made with
//    another device current is rejected with NMG_EINVAL (the scratch address
//    is per device).
#include <cuda_runtime.h>

#include "../../include/nmg.h"
#include "ctx.h"

static __device__ __align__(256) double g_noalloc_scratch[2 * NMG_NOALLOC_MAX_STATE];

namespace {
constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {nullptr};
}  // namespace

extern "C" int nmg_rk4_step_noalloc(nmg_ctx *c, double t, double dt, const double *u_in_dev,
                                    double *u_out_dev) {
  if (!c) return NMG_EINVAL;
  if (!u_in_dev || !u_out_dev || u_in_dev == u_out_dev)
    return nmg_ctx_fail_static(c, NMG_EINVAL,
                               "nmg_rk4_step_noalloc: u_in and u_out must be distinct device buffers");
  if (nmg_ctx_state_len(c) > (size_t)NMG_NOALLOC_MAX_STATE)
    return nmg_ctx_fail_static(c, NMG_EINVAL,
                               "nmg_rk4_step_noalloc: state larger than NMG_NOALLOC_MAX_STATE doubles");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return nmg_ctx_fail_static(c, NMG_ECUDA, "nmg_rk4_step_noalloc: no usable current device");
  if (dev != nmg_ctx_device(c))
    return nmg_ctx_fail_static(c, NMG_EINVAL,
                               "nmg_rk4_step_noalloc: the context's device is not the current device");
  if (!g_scratch_ptr[dev]) {
    // one-time set-up on this device (keep it outside stream capture)
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return nmg_ctx_fail_static(c, NMG_ECUDA,
                                 "nmg_rk4_step_noalloc: cudaGetSymbolAddress of the scratch failed");
    g_scratch_ptr[dev] = p;
  }
  double *s1 = g_scratch_ptr[dev];
  double *s2 = s1 + NMG_NOALLOC_MAX_STATE;
  return nmg_ctx_rk4_step_buffers(c, t, dt, u_in_dev, u_out_dev, s1, s2);
}
