// gs_common.cuh -- device helpers shared by the splat pipeline kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gs {

typedef uint32_t u32;
typedef uint64_t u64;

// Bits of the device error word (read back by gs_context_check / gs_sorter_check).
enum : u32 {
  ERR_CAPACITY = 1u,  // more (splat, tile) pairs than the context holds, or a sort count beyond max_count
  ERR_TIMEOUT = 2u,   // a bounded look-back wait gave up
  ERR_INTERNAL = 4u,  // a self-check failed (e.g. emitted tile pairs disagree with the counted ones)
};

// Upper bound on polls of one look-back status word.  A predecessor partition publishes its
// aggregate within microseconds of starting; a wait this long means it will never come, so the
// waiter records ERR_TIMEOUT and carries on with a zero contribution instead of hanging the GPU.
constexpr u32 kMaxSpins = 1u << 21;

__device__ __forceinline__ u64 ld_relaxed_u64(const u64* p) {
  u64 v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(u64* p, u64 v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ u32 lanemask_lt() {
  u32 m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Lanes of the warp whose 8-bit digit equals this lane's, among the lanes in `active` (8 ballots;
// faster than __match_any_sync on this architecture).  Must be called by the whole warp.
__device__ __forceinline__ u32 match_digit8(u32 d, bool active) {
  u32 peers = __ballot_sync(0xffffffffu, active);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1u;
    const u32 bb = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bb : ~bb;
  }
  return peers;
}

// Decoupled look-back status word: [63:32] epoch, [31:30] flag, [29:0] value.  A word whose epoch
// differs from the caller's is "not yet published" for this pass, so the status array never needs
// clearing between passes or frames.
enum : u32 { LB_AGGREGATE = 1u, LB_INCLUSIVE = 2u };

__device__ __forceinline__ u64 lb_pack(u32 epoch, u32 flag, u32 value) {
  return ((u64)epoch << 32) | ((u64)flag << 30) | (u64)(value & 0x3fffffffu);
}

// One thread's look-back for partition p over status words status[j * stride] (j < p).  Publishes
// `aggregate`, walks back until an inclusive prefix is found, publishes its own inclusive prefix and
// returns the exclusive prefix.  Every wait is bounded by kMaxSpins.
__device__ __forceinline__ void lb_publish(u64* status, u32 stride, u32 p, u32 epoch, u32 aggregate) {
  st_relaxed_u64(status + (size_t)p * stride, lb_pack(epoch, p == 0 ? LB_INCLUSIVE : LB_AGGREGATE, aggregate));
}

// The second half of lookback(), after lb_publish(aggregate): walks back, publishes the inclusive
// prefix and returns the exclusive one.
__device__ __forceinline__ u32 lb_resolve(u64* status, u32 stride, u32 p, u32 epoch, u32 aggregate, u32* err) {
  if (p == 0) return 0;
  u64* mine = status + (size_t)p * stride;
  u32 exclusive = 0;
  int j = (int)p - 1;
  u32 spins = 0;
  while (j >= 0) {
    const u64 s = ld_relaxed_u64(status + (size_t)j * stride);
    const u32 flag = (u32)(s >> 30) & 3u;
    if ((u32)(s >> 32) != epoch || flag == 0) {
      if (++spins > kMaxSpins) {
        atomicOr(err, ERR_TIMEOUT);
        break;
      }
      __nanosleep(32);
      continue;
    }
    exclusive += (u32)s & 0x3fffffffu;
    if (flag == LB_INCLUSIVE) break;
    --j;
  }
  st_relaxed_u64(mine, lb_pack(epoch, LB_INCLUSIVE, exclusive + aggregate));
  return exclusive;
}

// lb_resolve by a whole warp: lane l examines predecessor p-1-l (then 32 further back per step), so a
// walk over predecessors that have published only their aggregates costs one round trip per 32 of them.
// Every lane returns the exclusive prefix; lane 0 publishes the inclusive one.  Waits are bounded.
__device__ __forceinline__ u32 lb_resolve_warp(u64* status, u32 stride, u32 p, u32 epoch, u32 aggregate, u32* err) {
  const u32 lane = threadIdx.x & 31u;
  u32 exclusive = 0;
  for (int top = (int)p - 1; top >= 0; top -= 32) {
    const int j = top - (int)lane;
    u32 flag = LB_INCLUSIVE, value = 0;  // lanes beyond partition 0 stand for an empty inclusive prefix
    if (j >= 0) {
      u64 s = ld_relaxed_u64(status + (size_t)j * stride);
      for (u32 spins = 0; (u32)(s >> 32) != epoch || ((u32)(s >> 30) & 3u) == 0;) {
        if (++spins > kMaxSpins) {
          atomicOr(err, ERR_TIMEOUT);
          s = lb_pack(epoch, LB_INCLUSIVE, 0);
          break;
        }
        __nanosleep(32);
        s = ld_relaxed_u64(status + (size_t)j * stride);
      }
      flag = (u32)(s >> 30) & 3u;
      value = (u32)s & 0x3fffffffu;
    }
    const u32 incl = __ballot_sync(0xffffffffu, flag == LB_INCLUSIVE);
    const u32 stop = incl ? (u32)(__ffs(incl) - 1) : 31u;  // the nearest inclusive prefix ends the walk
    u32 v = lane <= stop ? value : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    exclusive += v;
    if (incl) break;
  }
  if (lane == 0 && p > 0) st_relaxed_u64(status + (size_t)p * stride, lb_pack(epoch, LB_INCLUSIVE, exclusive + aggregate));
  return exclusive;
}

__device__ __forceinline__ u32 lookback(u64* status, u32 stride, u32 p, u32 epoch, u32 aggregate, u32* err) {
  lb_publish(status, stride, p, epoch, aggregate);
  return lb_resolve(status, stride, p, epoch, aggregate, err);
}

// Exclusive scan of one value per thread across a block of NT threads (NT multiple of 32, <= 1024).
// Returns the exclusive prefix; *total receives the block sum.  Contains __syncthreads.
template <int NT>
__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32* s_warp /* >= NT/32 words */, u32* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    u32 w = (lane < NT / 32) ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NT / 32) s_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  const u32 before = warp ? s_warp[warp - 1] : 0u;
  *total = s_warp[NT / 32 - 1];
  __syncthreads();
  return before + x - v;
}

// Per-frame constants of one camera (the Camera uniform + model push constant, pre-multiplied
// where the reference multiplies per invocation).  Passed by value to the kernels.
// parse_ply.comp:62-88: cov3d = rot * diag(s^2) * rot^T from log-scales and a (x, y, z, w) quaternion of
// any length, in the shader's operation order (units including this must build without FMA contraction
// for the result to be the restatement's bits).  cov = (00, 10, 20, 11, 21, 22).
__device__ __forceinline__ void activate_cov3d(float ls0, float ls1, float ls2, float qx, float qy, float qz, float qw,
                                               float cov[6]) {
  const float s0 = expf(ls0), s1 = expf(ls1), s2 = expf(ls2);
  const float len = sqrtf(((qx * qx + qy * qy) + qz * qz) + qw * qw);
  qx = qx / len, qy = qy / len, qz = qz / len, qw = qw / len;
  const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
  const float xy = qx * qy, xz = qx * qz, yz = qy * qz;
  const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
  float R[3][3];  // rot[col][row], column-major as in the shader
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
  cov[0] = C(0, 0);
  cov[1] = C(1, 0);
  cov[2] = C(2, 0);
  cov[3] = C(1, 1);
  cov[4] = C(2, 1);
  cov[5] = C(2, 2);
}

__device__ __forceinline__ float activate_opacity(float logit) { return 1.0f / (1.0f + expf(-logit)); }

// Raster record of a splat: 4 float4 at record[4 * id].  The first two slots (32 bytes, one DRAM
// sector) hold everything the tile binning reads, so its random gathers touch one sector per splat.
enum : u32 {
  REC_CENTER = 0,  // (cx, cy, m00, m01): NDC centre (cx = +inf when the splat is not drawn), row 0 of M
  REC_AXES = 1,    // rot_scale columns (a.x, a.y, b.x, b.y): the 3-sigma quad is c +- 3a +- 3b
  REC_ROW1 = 2,    // (m10, m11, z, opacity): row 1 of M = rot_scale^-1, NDC depth, opacity
  REC_COLOR = 3,   // (r, g, b, drawn)
};

struct FrameConst {
  float pvm[16];    // projection * view * model, glm operand order (rank.comp:32)
  float model[16];
  float view[16];
  float proj[16];
  float cam_m[3];   // inverse(model) * camera_position, divided by w (projection.comp:85-86)
  float lpx, lpy;   // 1/W/W and 1/H/H (projection.comp:115-116)
  u32 width, height;
  u32 model_identity;
  u32 n;
};

}  // namespace gs
