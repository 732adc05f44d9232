// sm_103a kernels of the differentiable render and its adjoint (per-ray math
// in bh_adjoint_math.cuh).
//
// Schedule. A persistent grid (resident blocks only) walks the logical blocks
// of all scenes with a static stride; a logical block is 4 warps, each an
// 8x4 pixel tile of one scene, so neighbouring lanes trace neighbouring
// pixels (similar step counts and texture addresses). Each resident thread
// owns one checkpoint slot: ceil(max_steps / 64) checkpoints laid out
// [checkpoint][slot] so that a warp's stores are contiguous. The 8
// sub-checkpoints of the segment being reversed live in shared memory.
//
// Reduction. Per logical block the pixel losses and the 10 gradient terms
// are summed by warp shuffles and shared memory and added to the scene's FP64
// accumulators with one atomicAdd per value.
//
// MIXED. A classification kernel tests every ray's impact parameter in FP64
// and lists those with |b/M - 3 sqrt 3| < band; the band kernel traces the
// list (an FP64-accurate forward pass that keeps every state, an FP32 reverse
// pass over them) on a side stream while the main kernel traces the other
// rays in FP32. The main kernel takes its logical blocks from a queue.
#include <cuda_runtime.h>

#include <algorithm>

#include "bh_adjoint.h"
#include "bh_adjoint_math.cuh"

namespace bhgb {
namespace adj {
namespace {

constexpr int kThreads = 128;
// Dynamic shared memory of a band block (none: its reverse pass reads the
// stored trajectory through L1).
constexpr size_t kBandSmem = 0;
constexpr int kRed = kParams + 2;  // loss, gradient, steps
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int find_scene(const AdjLaunch& L, int64_t lb) {
  int lo = 0, hi = L.n_scenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (L.scenes[mid].block_begin <= lb) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void write_pixel(const AdjScene& s, int px, int py, const RayOut& o) {
  const size_t pix = (size_t)py * s.width + px;
  if (s.image) {
    s.image[pix * 3 + 0] = o.rgb[0];
    s.image[pix * 3 + 1] = o.rgb[1];
    s.image[pix * 3 + 2] = o.rgb[2];
  }
  if (s.pixel_grad) {
#pragma unroll
    for (int i = 0; i < kParams; ++i) s.pixel_grad[pix * kParams + i] = o.grad[i];
  }
}

// MIXED: appends every band ray (in_band) to the band list.
__global__ void adjoint_classify_kernel(AdjLaunch L) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < L.total_rays;
       r += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = L.n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (L.scenes[mid].ray_begin <= r) lo = mid;
      else hi = mid - 1;
    }
    const AdjScene& s = L.scenes[lo];
    const unsigned pix = unsigned(r - s.ray_begin);
    const int px = int(pix % unsigned(s.width)), py = int(pix / unsigned(s.width));
    if (in_band(s, px, py, L.p.band)) {
      const unsigned long long slot = atomicAdd(&L.counters[kCountBand], 1ull);
      if (slot < L.band_capacity) L.band_list[slot] = make_uint2(unsigned(lo), pix);
    }
  }
}

template <typename R, typename P, bool kComp, bool kDefer>
__global__ void __launch_bounds__(kThreads) adjoint_kernel(AdjLaunch L) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using CK = Ckpt<R, kComp>;
  CK* sub = reinterpret_cast<CK*>(smem_raw) + threadIdx.x;
  __shared__ float red[kThreads / 32][kRed];
  __shared__ long long next_block;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  CK* ck = static_cast<CK*>(L.ckpt) + (size_t)blockIdx.x * kThreads + tid;
  // logical blocks from a queue: blocks that start late (the band pass runs
  // beside this kernel) take fewer
  for (;;) {
    if (tid == 0) next_block = (long long)atomicAdd(&L.counters[kCountBlocks], 1ull);
    __syncthreads();
    const int64_t lb = next_block;
    if (lb >= L.total_blocks) break;
    const int sc = find_scene(L, lb);
    const AdjScene& s = L.scenes[sc];
    const int64_t tile = (lb - s.block_begin) * (kThreads / 32) + warp;
    const int px = int(tile % s.tiles_x) * 8 + (lane & 7);
    const int py = int(tile / s.tiles_x) * 4 + (lane >> 3);
    float v[kRed];
#pragma unroll
    for (int i = 0; i < kRed; ++i) v[i] = 0.f;
    if (px < s.width && py < s.height) {
      bool mine = true;
      RayC<R, P> rc;
      if constexpr (kDefer) mine = !in_band(s, px, py, L.p.band);  // traced by the band pass
      if (mine) {
        rc = ray_constants<R, P>(s, px, py, nullptr);
        RayOut o;
        trace_adjoint<R, P, kComp>(s, L.p, rc, px, py, ck, L.ckpt_slots, sub, kThreads, o);
        write_pixel(s, px, py, o);
        v[0] = o.loss;
#pragma unroll
        for (int i = 0; i < kParams; ++i) v[1 + i] = o.grad[i];
        v[kRed - 1] = float(o.steps);
      }
    }
#pragma unroll
    for (int i = 0; i < kRed; ++i) {
      float x = v[i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(kFull, x, off);
      if (lane == 0) red[warp][i] = x;
    }
    __syncthreads();
    if (tid < kRed) {
      float x = 0.f;
#pragma unroll
      for (int w = 0; w < kThreads / 32; ++w) x += red[w][tid];
      atomicAdd(&L.acc[(size_t)sc * kAccStride + (tid == kRed - 1 ? kAccSteps : tid)], double(x));
    }
    __syncthreads();
  }
}

// MIXED: the deferred rays. FP64 forward keeping every state; FP32 reverse
// pass over the kept states with compensated adjoint updates; the escape and
// crossing adjoints and the tangents in FP64 (trace_adjoint_band). Per-ray
// atomics: the list mixes scenes.
__global__ void __launch_bounds__(kThreads) adjoint_band_kernel(AdjLaunch L) {
  const int64_t slot = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  float2* traj = L.band_traj + slot;
  float* cross = L.band_cross + slot;
  double2* cross_xw = L.band_cross_xw + slot;
  const unsigned long long n = min(L.counters[kCountBand], (unsigned long long)L.band_capacity);
  if ((unsigned long long)blockIdx.x * kThreads >= n) return;
  for (unsigned long long i = (unsigned long long)slot; i < n; i += (unsigned long long)gridDim.x * kThreads) {
    const uint2 e = L.band_list[i];
    const AdjScene& s = L.scenes[e.x];
    const int px = int(e.y % (unsigned)s.width), py = int(e.y / (unsigned)s.width);
    RayOut o;
    trace_adjoint_band<float>(s, L.p, L.pband, px, py, traj, cross, cross_xw, L.band_slots, L.max_cross, o);
    write_pixel(s, px, py, o);
    double* acc = L.acc + (size_t)e.x * kAccStride;
    atomicAdd(acc, double(o.loss));
    for (int k = 0; k < kParams; ++k) atomicAdd(acc + 1 + k, double(o.grad[k]));
    atomicAdd(acc + kAccSteps, double(o.steps));
    atomicAdd(acc + kAccBandRays, 1.0);
  }
}

template <typename R, bool kComp>
constexpr size_t sub_bytes() {
  return sizeof(Ckpt<R, kComp>) * kThreads * (kSeg / kSub);
}

template <typename K>
cudaError_t prepare(K kernel, size_t smem, int sm_count, int64_t want, int* grid) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int64_t g = (int64_t)per_sm * sm_count;
  *grid = (int)(want < g ? (want < 1 ? 1 : want) : g);
  return cudaSuccess;
}

}  // namespace

size_t checkpoint_bytes(int precision) {
  if (precision == BH_PRECISION_FP64) return sizeof(Ckpt<double, false>);
  if (precision == BH_PRECISION_FP32) return sizeof(Ckpt<float, false>);
  return sizeof(Ckpt<float, true>);
}

cudaError_t plan_adjoint(int precision, int sm_count, int64_t total_blocks, int* main_grid, int* band_grid) {
  cudaError_t e;
  if (precision == BH_PRECISION_FP64)
    e = prepare(adjoint_kernel<double, double, false, false>, sub_bytes<double, false>(), sm_count, total_blocks,
                main_grid);
  else if (precision == BH_PRECISION_FP32)
    e = prepare(adjoint_kernel<float, float, false, false>, sub_bytes<float, false>(), sm_count, total_blocks,
                main_grid);
  else
    e = prepare(adjoint_kernel<float, double, true, true>, sub_bytes<float, true>(), sm_count, total_blocks,
                main_grid);
  if (e != cudaSuccess) return e;
  *band_grid = 0;
  if (precision == BH_PRECISION_MIXED) {
    // one block per SM: the band is a small fraction of the rays, and every
    // slot keeps a whole trajectory
    e = prepare(adjoint_band_kernel, kBandSmem, sm_count, total_blocks, band_grid);
    if (*band_grid > sm_count) *band_grid = sm_count;
  }
  return e;
}

cudaError_t launch_adjoint(const AdjLaunch& L, int main_grid, int band_grid, cudaStream_t st, cudaStream_t side,
                           cudaEvent_t ev_fork, cudaEvent_t ev_join) {
  cudaError_t e;
  if (L.precision == BH_PRECISION_MIXED) {
    // classify, then the band pass (long, latency-bound FP64-class rays) on
    // the side stream first and the main pass beside it
    const int cg = int(std::min<int64_t>((L.total_rays + 255) / 256, 4096));
    adjoint_classify_kernel<<<cg, 256, 0, st>>>(L);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev_fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(side, ev_fork, 0)) != cudaSuccess) return e;
    adjoint_band_kernel<<<band_grid, kThreads, kBandSmem, side>>>(L);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ev_join, side)) != cudaSuccess) return e;
    adjoint_kernel<float, double, true, true><<<main_grid, kThreads, sub_bytes<float, true>(), st>>>(L);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaStreamWaitEvent(st, ev_join, 0);
  }
  if (L.precision == BH_PRECISION_FP64)
    adjoint_kernel<double, double, false, false><<<main_grid, kThreads, sub_bytes<double, false>(), st>>>(L);
  else
    adjoint_kernel<float, float, false, false><<<main_grid, kThreads, sub_bytes<float, false>(), st>>>(L);
  return cudaGetLastError();
}

}  // namespace adj
}  // namespace bhgb
