// gs_ply.cu -- parse_ply.comp: activation of raw 3DGS PLY rows into the splat buffers, and the same
// activation of the differentiable path's raw parameters (k_activate).
//
// Follows src/shader/parse_ply.comp:43-97 with the row layout of splat_load_thread.cc:114-135
// (offsets[0..58] are float offsets inside a row, offsets[59] the row stride).  Compiled with
// --fmad=false so the covariance arithmetic keeps the shader's operation order; exp() is CUDA's
// correctly-rounded-within-2-ulp expf, so cov3d/opacity agree with a CPU restatement to a few ulps and
// the binary16 SH terms (round to nearest even) agree exactly.
#include <cuda_fp16.h>

#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

__global__ __launch_bounds__(256) void k_parse_ply(const float* __restrict__ rows, u32 count, const PlyOffsets off,
                                                   float* __restrict__ position, float* __restrict__ cov3d,
                                                   float* __restrict__ opacity, uint16_t* __restrict__ sh) {
  const u32 id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= count) return;
  const float* row = rows + (size_t)off.v[59] * id;
  float* cv = cov3d + 6 * (size_t)id;
  activate_cov3d(row[off.v[3]], row[off.v[4]], row[off.v[5]], row[off.v[6]], row[off.v[7]], row[off.v[8]],
                 row[off.v[9]], cv);
  position[3 * (size_t)id + 0] = row[off.v[0]];
  position[3 * (size_t)id + 1] = row[off.v[1]];
  position[3 * (size_t)id + 2] = row[off.v[2]];
  __half2* out = reinterpret_cast<__half2*>(sh + 48 * (size_t)id);
#pragma unroll
  for (int i = 0; i < 24; ++i) out[i] = __floats2half2_rn(row[off.v[10 + 2 * i]], row[off.v[11 + 2 * i]]);
  opacity[id] = activate_opacity(row[off.v[58]]);
}

cudaError_t launch_parse_ply(const float* rows, u32 count, const PlyOffsets& off, float* position, float* cov3d,
                             float* opacity, uint16_t* sh, cudaStream_t stream) {
  if (count == 0) return cudaSuccess;
  k_parse_ply<<<(count + 255) / 256, 256, 0, stream>>>(rows, count, off, position, cov3d, opacity, sh);
  return cudaGetLastError();
}

// parse_ply.comp's activation of the raw parameters (the same device code as k_parse_ply, so the records
// of the differentiable forward are the plain path's for the same splats); SH stay FP32.
__global__ void k_activate(const TrainArgs a) {
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 id = blockIdx.x * blockDim.x + threadIdx.x; id < a.n; id += stride) {
    const float4 q = reinterpret_cast<const float4*>(a.quats)[id];
    activate_cov3d(a.log_scales[3 * id], a.log_scales[3 * id + 1], a.log_scales[3 * id + 2], q.x, q.y, q.z, q.w,
                   a.cov3d + 6 * (size_t)id);
    a.opacity[id] = activate_opacity(a.opacity_logits[id]);
    a.position[3 * id] = a.means[3 * id];
    a.position[3 * id + 1] = a.means[3 * id + 1];
    a.position[3 * id + 2] = a.means[3 * id + 2];
  }
}

cudaError_t launch_activate(const TrainArgs& a, cudaStream_t stream) {
  if (a.n == 0) return cudaSuccess;
  k_activate<<<min((a.n + 255) / 256, 65535u), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace gs
