// Launch interface of the adjoint kernels (bh_adjoint.cu) for the C ABI
// (bh_capi.cu). Nothing here is part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bh_adjoint_math.cuh"

namespace bhgb {
namespace adj {

// device counters of one adjoint call
enum : int {
  kCountBand = 0,          // MIXED: rays appended to the band list
  kCountBandOverflow = 1,  // unused (the list holds every ray)
  kCountBlocks = 2,        // main pass work queue head (logical blocks)
  kCounters = 4
};

// per-scene accumulators: [0] sum of pixel losses, [1..10] gradient sums,
// [11] RK4 steps, [12] rays traced in the FP64 band pass
constexpr int kAccStride = 13;
constexpr int kAccSteps = 11;
constexpr int kAccBandRays = 12;

struct AdjLaunch {
  const AdjScene* scenes;
  int32_t n_scenes;
  int32_t precision;
  AdjParams p;
  int64_t total_blocks;   // logical blocks (4 tiles of 8x4 pixels) over all scenes
  void* ckpt;             // main pass checkpoints, [checkpoint][slot]
  int64_t ckpt_slots;     // main grid * threads
  AdjParams pband;        // MIXED band pass: the FP32 view of its FP64 trajectory
  float2* band_traj;      // band pass: every state, [step][slot]
  float* band_cross;      // band pass: transmittance before each crossing, [crossing][slot]
  double2* band_cross_xw; // band pass: FP64 state at each crossing, [crossing][slot]
  int32_t max_cross;
  int64_t band_slots;
  int64_t total_rays;     // all pixels of all scenes (classification)
  uint2* band_list;       // MIXED: (scene, pixel) of deferred rays
  uint32_t band_capacity;
  unsigned long long* counters;
  double* acc;
};

constexpr int kAdjThreads = 128;

size_t checkpoint_bytes(int precision);
// Resident grid sizes (capped at total_blocks) for a precision; sets the
// kernels' shared-memory attribute.
cudaError_t plan_adjoint(int precision, int sm_count, int64_t total_blocks, int* main_grid, int* band_grid);
// MIXED runs the band pass on side_stream concurrently with the main pass
// (fork and join through the two events).
cudaError_t launch_adjoint(const AdjLaunch& L, int main_grid, int band_grid, cudaStream_t stream,
                           cudaStream_t side_stream, cudaEvent_t ev_fork, cudaEvent_t ev_join);

}  // namespace adj
}  // namespace bhgb
