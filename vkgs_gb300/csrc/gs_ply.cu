// gs_ply.cu -- parse_ply.comp: activation of raw 3DGS PLY rows into the splat buffers.
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
  const float s0 = expf(row[off.v[3]]), s1 = expf(row[off.v[4]]), s2 = expf(row[off.v[5]]);
  float qx = row[off.v[6]], qy = row[off.v[7]], qz = row[off.v[8]], qw = row[off.v[9]];
  const float len = sqrtf(((qx * qx + qy * qy) + qz * qz) + qw * qw);
  qx = qx / len, qy = qy / len, qz = qz / len, qw = qw / len;
  const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
  const float xy = qx * qy, xz = qx * qz, yz = qy * qz;
  const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
  // rot[col][row], column-major as in the shader
  float R[3][3];
  R[0][0] = 1.0f - 2.0f * (yy + zz);
  R[0][1] = 2.0f * (xy + wz);
  R[0][2] = 2.0f * (xz - wy);
  R[1][0] = 2.0f * (xy - wz);
  R[1][1] = 1.0f - 2.0f * (xx + zz);
  R[1][2] = 2.0f * (yz + wx);
  R[2][0] = 2.0f * (xz + wy);
  R[2][1] = 2.0f * (yz - wx);
  R[2][2] = 1.0f - 2.0f * (xx + yy);
  const float S[3] = {s0 * s0, s1 * s1, s2 * s2};
  // (rot * diag(S)) has columns S[j] * rot[j]; the shader's full product adds exact zeros, which
  // leave every nonzero sum unchanged.
  float T[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) T[j][i] = R[j][i] * S[j];
  // cov = T * rot^T: cov[j][i] = (T[0][i] rot[0][j] + T[1][i] rot[1][j]) + T[2][i] rot[2][j]
  const auto C = [&](int j, int i) { return (T[0][i] * R[0][j] + T[1][i] * R[1][j]) + T[2][i] * R[2][j]; };
  float* cv = cov3d + 6 * (size_t)id;
  cv[0] = C(0, 0);
  cv[1] = C(1, 0);
  cv[2] = C(2, 0);
  cv[3] = C(1, 1);
  cv[4] = C(2, 1);
  cv[5] = C(2, 2);
  position[3 * (size_t)id + 0] = row[off.v[0]];
  position[3 * (size_t)id + 1] = row[off.v[1]];
  position[3 * (size_t)id + 2] = row[off.v[2]];
  __half2* out = reinterpret_cast<__half2*>(sh + 48 * (size_t)id);
#pragma unroll
  for (int i = 0; i < 24; ++i) out[i] = __floats2half2_rn(row[off.v[10 + 2 * i]], row[off.v[11 + 2 * i]]);
  opacity[id] = 1.0f / (1.0f + expf(-row[off.v[58]]));
}

cudaError_t launch_parse_ply(const float* rows, u32 count, const PlyOffsets& off, float* position, float* cov3d,
                             float* opacity, uint16_t* sh, cudaStream_t stream) {
  if (count == 0) return cudaSuccess;
  k_parse_ply<<<(count + 255) / 256, 256, 0, stream>>>(rows, count, off, position, cov3d, opacity, sh);
  return cudaGetLastError();
}

}  // namespace gs
