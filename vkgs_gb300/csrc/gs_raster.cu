// gs_raster.cu -- 16x16-tile rasteriser + blend, the CUDA form of the reference's quad draw.
//
// Reference semantics (splat.vert:10-25, splat.frag:8-12, engine.cc:281-300, 1382-1387):
//   * a splat covers a pixel iff the pixel centre lies in its 3-sigma quad; in the quad's unit frame
//     p = rot_scale^-1 (ndc - center) that is |p.x| <= 3 and |p.y| <= 3;
//   * fragment alpha a = opacity * exp(-0.5 |p|^2), colour clamped to [0,1] like a UNORM attachment;
//   * depth test LESS against the cleared 1.0 (or a caller depth buffer), no depth write;
//   * blend RGB <- a*rgb + (1-a)*RGB and A <- a*a + (1-a)*A over (0,0,0,1), in ascending sorted order
//     (far to near).
// Here each pixel accumulates the same sum front to back: RGB = sum a_i rgb_i T_i,
// A = sum a_i^2 T_i + T_end, T_i = prod_{j nearer} (1 - a_j).  The coverage arithmetic uses
// explicitly rounded operations (no FMA) so that the set of covered (pixel, splat) pairs is exactly
// the restatement's.  A tile stops once every pixel's transmittance is below t_floor: the splats
// behind can then change no channel by more than t_floor.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

constexpr int kRasterThreads = kTile * kTile;  // one pixel per thread

template <bool DEPTH, bool COUNT>
__global__ __launch_bounds__(kRasterThreads) void k_raster(const RasterArgs a) {
  __shared__ float4 s_q0[kRasterThreads];  // cx, cy, m00, m01
  __shared__ float4 s_q1[kRasterThreads];  // m10, m11, cz, opacity
  __shared__ float4 s_q2[kRasterThreads];  // r, g, b, -
  const u32 tile = blockIdx.x;
  const u32 tx = tile % a.tiles_x, ty = tile / a.tiles_x;
  const u32 tid = threadIdx.x;
  const u32 px = tx * kTile + (tid % kTile), py = ty * kTile + (tid / kTile);
  const bool inside = px < a.width && py < a.height;
  const float fx = __fdiv_rn((float)(2 * px + 1), (float)a.width) - 1.0f;
  const float fy = __fdiv_rn((float)(2 * py + 1), (float)a.height) - 1.0f;
  const float dpix = (DEPTH && inside) ? a.depth[(size_t)py * a.width + px] : 1.0f;
  const uint2 tr = reinterpret_cast<const uint2*>(a.tile_range)[tile];
  const uint2 range = make_uint2(min(tr.x, a.pair_capacity), min(tr.y, a.pair_capacity));

  float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f, ca = 0.0f;
  u32 frags = 0, needed = 0;
  const float kExp = -0.5f * 1.4426950408889634f;  // -log2(e)/2
  bool done = !inside;
  for (u32 hi = range.y; hi > range.x;) {
    const u32 lo = (hi - range.x > (u32)kRasterThreads) ? hi - kRasterThreads : range.x;
    const u32 cnt = hi - lo;
    if (tid < cnt) {
      const u32 id = a.pair_splat[hi - 1 - tid];  // nearest first
      const float4* rec = a.record + 4 * (size_t)id;
      s_q0[tid] = rec[0];
      s_q1[tid] = rec[1];
      s_q2[tid] = rec[2];
    }
    __syncthreads();
    if (!__all_sync(0xffffffffu, done)) {
      for (u32 j = 0; j < cnt; ++j) {
        const float4 q0 = s_q0[j], q1 = s_q1[j];
        const float dx = __fsub_rn(fx, q0.x), dy = __fsub_rn(fy, q0.y);
        const float u = __fadd_rn(__fmul_rn(q0.z, dx), __fmul_rn(q0.w, dy));
        const float v = __fadd_rn(__fmul_rn(q1.x, dx), __fmul_rn(q1.y, dy));
        bool cov = (fabsf(u) <= 3.0f) & (fabsf(v) <= 3.0f);
        if (DEPTH) cov &= q1.z < dpix;
        if (COUNT) {
          frags += (cov && inside) ? 1u : 0u;
          needed += (cov && inside && T >= a.t_floor) ? 1u : 0u;
        }
        const float g = exp2f(kExp * (u * u + v * v));
        const float al = cov ? q1.w * g : 0.0f;
        const float w = al * T;
        const float4 q2 = s_q2[j];
        cr += w * q2.x;
        cg += w * q2.y;
        cb += w * q2.z;
        ca += w * al;
        T -= w;
      }
    }
    hi = lo;
    if (!COUNT) done = done || T < a.t_floor;
    // Barrier before the next batch overwrites shared memory; also ends the tile once all are done.
    if (__syncthreads_and(done)) break;
  }
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      frags += __shfl_xor_sync(0xffffffffu, frags, o);
      needed += __shfl_xor_sync(0xffffffffu, needed, o);
    }
    if ((tid & 31) == 0 && frags) atomicAdd(a.fragments, (unsigned long long)frags);
    if ((tid & 31) == 0 && needed) atomicAdd(a.fragments + 1, (unsigned long long)needed);
  }
  if (!inside) return;
  const size_t pix = (size_t)py * a.width + px;
  const float alpha = ca + T;
  if (a.out_rgba) reinterpret_cast<float4*>(a.out_rgba)[pix] = make_float4(cr, cg, cb, alpha);
  if (a.out_bgra) {
    const auto q = [](float x) { return (unsigned char)__float2uint_rn(__saturatef(x) * 255.0f); };
    a.out_bgra[pix] = make_uchar4(q(cb), q(cg), q(cr), q(alpha));
  }
}

cudaError_t launch_raster(const RasterArgs& a, cudaStream_t stream) {
  const u32 tiles = a.tiles_x * a.tiles_y;
  if (tiles == 0) return cudaSuccess;
  const bool depth = a.depth != nullptr, count = a.fragments != nullptr;
  if (depth && count)
    k_raster<true, true><<<tiles, kRasterThreads, 0, stream>>>(a);
  else if (depth)
    k_raster<true, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  else if (count)
    k_raster<false, true><<<tiles, kRasterThreads, 0, stream>>>(a);
  else
    k_raster<false, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace gs
