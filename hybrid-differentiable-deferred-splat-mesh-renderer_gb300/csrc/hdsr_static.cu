// hdsr_static.cu — hdsr_count_tile_refs_static: per-tile splat counts of a
// projected frame without any device allocation.
//
// The same counts as the handle's tile-count stage (the 2D difference grid of
// hdsr_project.cu, the counts of count_tile_refs in
// gpu_tile_splat_composite.wgsl:65-84), but the difference grid lives in a
// file-scope __device__ array instead of a handle buffer, so the call needs
// no handle and allocates nothing:
//   - scratch: kStaticDiffWords ints (256 KiB), enough for every tile grid a
//     plan accepts (<= 255 x 255 tiles -> <= 256 x 256 grid words); larger
//     grids are rejected with HDSR_ERR_UNSUPPORTED before any device work;
//   - set-up: the first call on a device, with that device current, looks
//     the array's device address up once (cudaGetSymbolAddress) and keeps it
//     per device; that first call should come before any stream capture.
//     The kept address belongs to the device's primary context: after
//     cudaDeviceReset it is stale, so callers must not use the entry point
//     again in that process;
//   - nothing has to start at zero: every call zeroes the grid words it uses
//     and the whole output in its first kernel;
//   - calls on one device share the scratch: two calls whose kernels overlap
//     in time (different streams, no ordering between them) race on it.
#include <cstdio>
#include <mutex>

#include "../../include/hdsr.h"
#include "hdsr_internal.cuh"

namespace hdsr {
namespace {

constexpr uint32_t kStaticDiffWords = 256u * 256u;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) int g_static_diff[kStaticDiffWords];

std::mutex g_static_mu;
int* g_static_ptr[kStaticMaxDevices] = {};

__global__ void k_static_zero(int* diff, uint32_t n, uint32_t* counts, uint64_t len) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) diff[i] = 0;
  if (i < len) counts[i] = 0u;
}

__global__ void k_static_diff(const uint32_t* boxes, uint32_t stride, uint64_t n, int* diff, uint32_t gstride,
                              uint32_t cols, uint32_t rows) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint32_t box = boxes[r * stride];
  if (box == kSentinel) return;
  const uint32_t x0 = box & 0xFFu, y0 = (box >> 8) & 0xFFu, x1 = ((box >> 16) & 0xFFu) + 1u, y1 = (box >> 24) + 1u;
  if (x0 >= x1 || y0 >= y1 || x1 > cols || y1 > rows) return;  // not a box of this grid
  atomicAdd(diff + y0 * gstride + x0, 1);
  atomicAdd(diff + y0 * gstride + x1, -1);
  atomicAdd(diff + y1 * gstride + x0, -1);
  atomicAdd(diff + y1 * gstride + x1, 1);
}

// One block: row prefixes, then column prefixes written in Morton order.
__global__ void __launch_bounds__(256) k_static_prefix(int* diff, uint32_t gstride, uint32_t cols, uint32_t rows,
                                                       uint32_t* counts) {
  for (uint32_t y = threadIdx.x; y < rows; y += blockDim.x) {
    int run = 0;
    for (uint32_t x = 0; x < cols; ++x) {
      run += diff[y * gstride + x];
      diff[y * gstride + x] = run;
    }
  }
  __syncthreads();
  for (uint32_t x = threadIdx.x; x < cols; x += blockDim.x) {
    int run = 0;
    for (uint32_t y = 0; y < rows; ++y) {
      run += diff[y * gstride + x];
      counts[morton(x, y)] = (uint32_t)run;
    }
  }
}

}  // namespace
}  // namespace hdsr

using namespace hdsr;

extern "C" hdsr_status hdsr_count_tile_refs_static(const uint32_t* tile_boxes, uint32_t box_stride_words,
                                                   uint64_t splat_count, uint32_t tile_columns,
                                                   uint32_t tile_rows, uint32_t* tile_counts,
                                                   uint64_t tile_counts_len, void* stream) {
  if (tile_columns == 0u || tile_rows == 0u || box_stride_words == 0u || !tile_counts) return HDSR_ERR_INVALID_ARG;
  if (splat_count && !tile_boxes) return HDSR_ERR_INVALID_ARG;
  if (tile_columns > 255u || tile_rows > 255u ||
      (uint64_t)(tile_columns + 1u) * (tile_rows + 1u) > kStaticDiffWords)
    return HDSR_ERR_UNSUPPORTED;  // grid larger than the static scratch
  if (tile_counts_len < (uint64_t)morton(tile_columns - 1u, tile_rows - 1u) + 1u) return HDSR_ERR_INVALID_ARG;
  if (tile_counts_len >= (1ull << 32) || splat_count >= (1ull << 32)) return HDSR_ERR_UNSUPPORTED;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices) return HDSR_ERR_CUDA;
  int* diff = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_diff) != cudaSuccess || !p) return HDSR_ERR_CUDA;
      g_static_ptr[dev] = static_cast<int*>(p);
    }
    diff = g_static_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint32_t gstride = tile_columns + 1u, words = gstride * (tile_rows + 1u);
  const uint64_t zn = words > tile_counts_len ? words : tile_counts_len;
  k_static_zero<<<(unsigned)((zn + 255u) / 256u), 256, 0, s>>>(diff, words, tile_counts, tile_counts_len);
  if (splat_count)
    k_static_diff<<<(unsigned)((splat_count + 255u) / 256u), 256, 0, s>>>(tile_boxes, box_stride_words, splat_count,
                                                                          diff, gstride, tile_columns, tile_rows);
  k_static_prefix<<<1, 256, 0, s>>>(diff, gstride, tile_columns, tile_rows, tile_counts);
  return cudaGetLastError() == cudaSuccess ? HDSR_OK : HDSR_ERR_CUDA;
}
