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
  kCountBandOverflow = 1,  // band rays kept in FP32 because the list was full
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
  void* ckpt_band;        // MIXED band pass checkpoints
  int64_t band_slots;
  uint2* band_list;       // MIXED: (scene, pixel) of deferred rays
  uint32_t band_capacity;
  unsigned long long* counters;
  double* acc;
};

constexpr int kAdjThreads = 128;

size_t checkpoint_bytes(int precision);
size_t band_checkpoint_bytes();
// Resident grid sizes (capped at total_blocks) for a precision; sets the
// kernels' shared-memory attribute.
cudaError_t plan_adjoint(int precision, int sm_count, int64_t total_blocks, int* main_grid, int* band_grid);
cudaError_t launch_adjoint(const AdjLaunch& L, int main_grid, int band_grid, cudaStream_t stream);

}  // namespace adj
}  // namespace bhgb
