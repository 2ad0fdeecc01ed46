// hdsr_backward_prep.cu — first kernel of the frame's adjoint: per sortRank,
// the screen-space parameters the adjoint rasteriser composites with
// (centre, conic, clamped opacity with the anti-aliasing factor, clamped SH
// colour), computed without the f16 rounding of the cache and with the
// cancellation-free conic, then stored at fp32; zeroes the screen-space
// gradient accumulators. The recompute runs in double-float (hdsr_df64.cuh,
// about 44 bits; -DHDSR_BWD_REAL=double selects fp64): for a splat seen nearly
// edge-on, fp32 rounding of b0 and b1 is amplified by 1 / sin(angle between
// them) in |b0 x b1|^2, and its opacity (through the anti-aliasing factor)
// and conic then miss the FP64 ones by up to about 1%.
#ifndef HDSR_BWD_REAL
#define HDSR_BWD_REAL df64
#endif
#include "hdsr_proj_adjoint.cuh"

namespace hdsr {
namespace {

__global__ void __launch_bounds__(256) k_bwd_prep(BwdArgs b) {
  const FrameArgs& a = b.f;
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.N) return;
#pragma unroll
  for (uint32_t j = 0; j < kG2d; ++j) b.g2d[(size_t)r * kG2d + j] = 0.0f;
  float4* par = b.par + (size_t)r * 3;
  if (a.aux[r].x == kSentinel) {
    par[0] = par[1] = par[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  Proj P;
  proj_recompute(a, __ldg(a.sorted + r), P);
  const real Di = 1.0f / P.D;
  par[0] = make_float4(to_float(P.cx), to_float(P.cy), to_float(P.cYY * Di), to_float(-P.XY * Di));
  par[1] = make_float4(to_float(P.cXX * Di), to_float(rclamp_(P.op_aa, 0.0f, 0.99f)),
                       to_float(rclamp_(P.craw[0], 0.0f, 1.0f)), to_float(rclamp_(P.craw[1], 0.0f, 1.0f)));
  par[2] = make_float4(to_float(rclamp_(P.craw[2], 0.0f, 1.0f)), 0.0f, 0.0f, 0.0f);
}

}  // namespace

cudaError_t launch_bwd_prep(const BwdArgs& b, cudaStream_t s) {
  if (b.f.N) k_bwd_prep<<<(b.f.N + 255) / 256, 256, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace hdsr
