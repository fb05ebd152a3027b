// gs_cull.cu -- rank.comp + projection.comp fused into one pass over the splats in id order.
//
// Compiled with --fmad=false: every product and sum below is one IEEE binary32 rounding in the
// operand order of the GLSL source (column-major matrices, left-to-right sums), so the visible set,
// the keys and the projected records are bit-identical to the scalar restatement of the shaders.
//
// Per 1024-splat partition (partitions taken in ticket order by persistent CTAs):
//   1. rank.comp:27-41 -- clip = (P*V*M) * pos, ndc = clip / clip.w, visible iff |x|<=1, |y|<=1,
//      0<=z<=1, key = floatBitsToUint(1 - z);
//   2. the reference's atomicAdd slot becomes an order-preserving compaction (ballot counts per warp,
//      a bounded decoupled look-back across partitions), so equal keys later sort by ascending id;
//      the partition publishes its count at once and resolves its own offset only after step 3;
//   3. projection.comp:80-179 for every visible splat, written at record[id] (raster record) and,
//      if requested, inst_by_id[id] (the reference's 48-byte instance layout);
//   4. the keys and ids are written at their compacted slots.
// The reference's inverse-index pass (inverse_index.comp) has no counterpart: records are keyed by
// splat id and the later stages gather them through the sorted index list.
#include <cuda_fp16.h>

#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

__device__ __forceinline__ void mat4_vec4(const float* m, const float v[4], float out[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i] = ((m[i] * v[0] + m[4 + i] * v[1]) + m[8 + i] * v[2]) + m[12 + i] * v[3];
}

// cov <- m3 * cov * transpose(m3), m3 = mat3(m4), evaluated as (m3 * cov) * m3^T, all 9 entries.
__device__ __forceinline__ void sandwich3(const float* m4, float c[9]) {
  float t[9];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      t[j * 3 + i] = (m4[0 * 4 + i] * c[j * 3 + 0] + m4[1 * 4 + i] * c[j * 3 + 1]) + m4[2 * 4 + i] * c[j * 3 + 2];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      c[j * 3 + i] = (t[0 * 3 + i] * m4[0 * 4 + j] + t[1 * 3 + i] * m4[1 * 4 + j]) + t[2 * 3 + i] * m4[2 * 4 + j];
}

__device__ __forceinline__ float dot4(float a0, float a1, float a2, float a3, float b0, float b1, float b2, float b3) {
  return ((a0 * b0 + a1 * b1) + a2 * b2) + a3 * b3;
}

__device__ __forceinline__ void unpack_half8(const uint4 q, float f[8]) {
  const __half2* h = reinterpret_cast<const __half2*>(&q);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 v = __half22float2(h[i]);
    f[2 * i] = v.x;
    f[2 * i + 1] = v.y;
  }
}

// SH32: FP32 coefficients (the differentiable path) instead of binary16 -- a separate instantiation, so
// the plain path's kernel keeps its register count.
template <bool SH32>
__device__ void project_splat(const FrameConst& fc, const CullArgs& a, u32 id, float x0, float y0, float z0) {
  // direction for SH in model space (projection.comp:85-87); normalize = v / sqrt(dot(v, v))
  const float ddx = x0 - fc.cam_m[0], ddy = y0 - fc.cam_m[1], ddz = z0 - fc.cam_m[2];
  const float dl = sqrtf((ddx * ddx + ddy * ddy) + ddz * ddz);
  const float x = ddx / dl, y = ddy / dl, z = ddz / dl;

  const float* cv = a.cov3d + 6 * (size_t)id;
  const float c0 = __ldg(cv + 0), c1 = __ldg(cv + 1), c2 = __ldg(cv + 2), c3 = __ldg(cv + 3), c4 = __ldg(cv + 4),
              c5 = __ldg(cv + 5);
  float C[9] = {c0, c1, c2, c1, c3, c4, c2, c4, c5};  // mat3(v0, v0.y, v1.xy, v0.z, v1.yz)
  float p4[4] = {x0, y0, z0, 1.0f};
  if (!fc.model_identity) {
    sandwich3(fc.model, C);
    float t[4];
    mat4_vec4(fc.model, p4, t);
    p4[0] = t[0], p4[1] = t[1], p4[2] = t[2], p4[3] = t[3];
  }
  sandwich3(fc.view, C);
  float pv[4];
  mat4_vec4(fc.view, p4, pv);

  // J (projection.comp:105-108); only its first two rows reach the 2x2 block, and the
  // structural zeros J[1][0] = J[0][1] = 0 contribute exact zeros to every sum they enter.
  const float j00 = -1.0f / pv[2];
  const float j20 = pv[0] / pv[2] / pv[2];
  const float j21 = pv[1] / pv[2] / pv[2];
  float jc0[3], jc1[3];  // (J * C)[k][0], (J * C)[k][1]
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    jc0[k] = j00 * C[k * 3 + 0] + j20 * C[k * 3 + 2];
    jc1[k] = j00 * C[k * 3 + 1] + j21 * C[k * 3 + 2];
  }
  const float r00 = jc0[0] * j00 + jc0[2] * j20;  // (J C J^T)[0][0]
  const float r01 = jc1[0] * j00 + jc1[2] * j20;  // [0][1]
  const float r10 = jc0[1] * j00 + jc0[2] * j21;  // [1][0]
  const float r11 = jc1[1] * j00 + jc1[2] * j21;  // [1][1]

  // cov2d = mat2(P) * mat2(cov) * mat2(P) (projection.comp:111-112)
  const float p00 = fc.proj[0], p01 = fc.proj[1], p10 = fc.proj[4], p11 = fc.proj[5];
  const float t00 = p00 * r00 + p10 * r01, t01 = p01 * r00 + p11 * r01;
  const float t10 = p00 * r10 + p10 * r11, t11 = p01 * r10 + p11 * r11;
  const float a2 = (t00 * p00 + t10 * p01) + fc.lpx;
  const float b2 = (t01 * p10 + t11 * p11) + fc.lpy;
  const float c2d = t00 * p10 + t10 * p11;

  // eigen decomposition (projection.comp:121-134); the angle through the half-angle identities
  const float D = sqrtf((a2 - b2) * (a2 - b2) + 4.0f * c2d * c2d);
  const float s0 = sqrtf(0.5f * (a2 + b2 + D));
  const float s1 = sqrtf(0.5f * (a2 + b2 - D));
  const float sin2t = 2.0f * c2d / D;
  const float cos2t = (a2 - b2) / D;
  float ct, st;
  if (cos2t >= 0.0f) {
    ct = sqrtf(0.5f * (1.0f + cos2t));
    st = sin2t / (2.0f * ct);
  } else {
    const float s = sqrtf(0.5f * (1.0f - cos2t));
    st = copysignf(s, sin2t);
    ct = fabsf(sin2t) / (2.0f * s);
  }
  const float rs0 = s0 * ct, rs1 = s0 * st, rs2 = -s1 * st, rs3 = s1 * ct;

  // ndc (projection.comp:136-137)
  float pc[4];
  mat4_vec4(fc.proj, pv, pc);
  const float nx = pc[0] / pc[3], ny = pc[1] / pc[3], nz = pc[2] / pc[3];

  // SH degree 3 (projection.comp:140-174)
  const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f, C20 = 1.0925484305920792f,
              C21 = 0.31539156525252005f, C22 = 0.5462742152960396f, C30 = 0.5900435899266435f,
              C31 = 2.890611442640554f, C32 = 0.4570457994644658f, C33 = 0.3731763325901154f,
              C34 = 1.445305721320277f;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  const float b00 = C0, b01 = -C1 * y, b02 = C1 * z, b03 = -C1 * x;
  const float b10 = C20 * xy, b11 = -C20 * yz, b12 = C21 * (2.0f * zz - xx - yy), b13 = -C20 * xz;
  const float b20 = C22 * (xx - yy), b21 = -C30 * y * (3.0f * xx - yy), b22 = C31 * xy * z,
              b23 = -C32 * y * (4.0f * zz - xx - yy);
  const float b30 = C33 * z * (2.0f * zz - 3.0f * xx - 3.0f * yy), b31 = -C32 * x * (4.0f * zz - xx - yy),
              b32 = C34 * z * (xx - yy), b33 = -C30 * x * (xx - 3.0f * yy);
  const uint4* shv = reinterpret_cast<const uint4*>(a.sh + 48 * (size_t)id);
  const float4* sh32 = SH32 ? reinterpret_cast<const float4*>(a.sh32 + 48 * (size_t)id) : nullptr;
  float color[3];
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    float g[16];
    if (SH32) {  // FP32 coefficients (the differentiable path)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float4 v = __ldg(sh32 + 4 * ch + k);
        g[4 * k] = v.x, g[4 * k + 1] = v.y, g[4 * k + 2] = v.z, g[4 * k + 3] = v.w;
      }
    } else {
      unpack_half8(__ldg(shv + 2 * ch), g);
      unpack_half8(__ldg(shv + 2 * ch + 1), g + 8);
    }
    const float col = ((dot4(b00, b01, b02, b03, g[0], g[1], g[2], g[3]) +
                        dot4(b10, b11, b12, b13, g[4], g[5], g[6], g[7])) +
                       dot4(b20, b21, b22, b23, g[8], g[9], g[10], g[11])) +
                      dot4(b30, b31, b32, b33, g[12], g[13], g[14], g[15]);
    color[ch] = fmaxf(col + 0.5f, 0.0f);
  }
  const float o = __ldg(a.opacity + id);

  const float m00 = ct / s0, m01 = st / s0, m10 = -st / s1, m11 = ct / s1;
  const bool drawn = (s1 > 0.0f) && isfinite(m00) && isfinite(m01) && isfinite(m10) && isfinite(m11) &&
                     (nz >= 0.0f) && (nz < 1.0f);
  float4* rec = a.record + 4 * (size_t)id;
  rec[REC_CENTER] = make_float4(drawn ? nx : INFINITY, ny, m00, m01);  // +inf: the binning skips it
  rec[REC_AXES] = make_float4(rs0, rs1, rs2, rs3);
  rec[REC_ROW1] = make_float4(m10, m11, nz, o);
  rec[REC_COLOR] = make_float4(fminf(color[0], 1.0f), fminf(color[1], 1.0f), fminf(color[2], 1.0f), drawn ? 1.0f : 0.0f);
  if (a.inst_by_id) {
    float4* inst = reinterpret_cast<float4*>(a.inst_by_id + 12 * (size_t)id);
    inst[0] = make_float4(nx, ny, nz, 0.0f);
    inst[1] = make_float4(rs0, rs1, rs2, rs3);
    inst[2] = make_float4(color[0], color[1], color[2], o);
  }
}

template <bool SH32>
__global__ __launch_bounds__(kCullThreads, 6) void k_cull_project(const FrameConst fc, const CullArgs a) {
  __shared__ u32 s_cnt[kCullItems][kCullThreads / 32];
  __shared__ u32 s_off[kCullItems][kCullThreads / 32];
  __shared__ u32 s_key[kCullItems][kCullThreads];  // keys wait here while the partition projects
  __shared__ u32 s_base, s_acc;
  __shared__ u32 s_part;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 n = fc.n;
  const u32 nparts = (n + kCullTile - 1) / kCullTile;
  for (;;) {
    if (tid == 0) s_part = atomicAdd(a.ticket, 1u);
    __syncthreads();
    const u32 p = s_part;
    if (p >= nparts) break;
    float px[kCullItems], py[kCullItems], pz[kCullItems];
    bool vis[kCullItems];
#pragma unroll
    for (u32 k = 0; k < kCullItems; ++k) {
      const u32 id = p * kCullTile + k * kCullThreads + tid;
      vis[k] = false;
      px[k] = py[k] = pz[k] = 0.0f;
      if (id < n) {
        px[k] = __ldg(a.position + 3 * (size_t)id + 0);
        py[k] = __ldg(a.position + 3 * (size_t)id + 1);
        pz[k] = __ldg(a.position + 3 * (size_t)id + 2);
        const float v[4] = {px[k], py[k], pz[k], 1.0f};
        float c[4];
        mat4_vec4(fc.pvm, v, c);
        const float x = c[0] / c[3], y = c[1] / c[3], z = c[2] / c[3];
        vis[k] = fabsf(x) <= 1.0f && fabsf(y) <= 1.0f && z >= 0.0f && z <= 1.0f;
        s_key[k][tid] = __float_as_uint(1.0f - z);
      }
      const u32 ball = __ballot_sync(0xffffffffu, vis[k]);
      if (lane == 0) s_cnt[k][warp] = __popc(ball);
    }
    __syncthreads();
    // The partition's aggregate is published at once; its look-back is resolved after the projection
    // (which writes by id and needs no offset), so the wait overlaps with work.  What the key writes
    // need afterwards is re-read from shared memory, so little stays live across the projection calls.
    if (tid == 0) {
      u32 acc = 0;
      for (u32 k = 0; k < kCullItems; ++k)
        for (u32 w = 0; w < kCullThreads / 32; ++w) {
          s_off[k][w] = acc;
          acc += s_cnt[k][w];
        }
      s_acc = acc;
      lb_publish(a.status, 1, p, a.epoch, acc);
    }
    {
      const u32 id0 = p * kCullTile + tid;
#pragma unroll 1
      for (u32 k = 0; k < kCullItems; ++k)
        if (vis[k]) project_splat<SH32>(fc, a, id0 + k * kCullThreads, px[k], py[k], pz[k]);
    }
    const u32 t = threadIdx.x, pp = *reinterpret_cast<volatile u32*>(&s_part);
    if (t == 0) {
      const u32 acc = s_acc;
      const u32 excl = lb_resolve(a.status, 1, pp, a.epoch, acc, a.err);
      s_base = excl;
      if (pp == nparts - 1) *a.visible_count = excl + acc;
    }
    __syncthreads();
    const u32 ltm = lanemask_lt();
#pragma unroll
    for (u32 k = 0; k < kCullItems; ++k) {
      const u32 ball = __ballot_sync(0xffffffffu, vis[k]);
      if (vis[k]) {
        const u32 slot = s_base + s_off[k][t >> 5] + __popc(ball & ltm);
        a.key[slot] = s_key[k][t];
        a.index[slot] = pp * kCullTile + k * kCullThreads + t;
      }
    }
    __syncthreads();
  }
}

// Many views of the same splats in one pass (the batched form): each partition's positions are loaded
// once, every view's visibility and ballots are taken from them, thread v of the first warp publishes
// and later resolves view v's look-back, each visible (splat, view) is projected into that view's
// records, and then keyed into its compacted lists.
// The splat's covariance, opacity and SH are read once per partition from DRAM and then from cache for
// the other views.  Outputs are bit-identical to k_cull_project<SH32> run per view.
template <bool SH32>
__global__ __launch_bounds__(kCullThreads) void k_cull_views(const CullViewsArgs a) {
  __shared__ u32 s_cnt[kMaxCullViews][kCullItems][kCullThreads / 32];
  __shared__ u32 s_base[kMaxCullViews], s_acc[kMaxCullViews];
  __shared__ u32 s_part;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 n = a.n, nv = a.count;
  const u32 nparts = (n + kCullTile - 1) / kCullTile;
  const u32 lt = lanemask_lt();
  CullArgs ca{};  // the shared inputs; the record pointer is set per view
  ca.position = a.position;
  ca.cov3d = a.cov3d;
  ca.opacity = a.opacity;
  ca.sh = a.sh;
  ca.sh32 = a.sh32;
  for (;;) {
    if (tid == 0) s_part = atomicAdd(a.ticket, 1u);
    __syncthreads();
    const u32 p = s_part;
    if (p >= nparts) break;
    float px[kCullItems], py[kCullItems], pz[kCullItems];
    u32 visbits[kCullItems];
#pragma unroll
    for (u32 k = 0; k < kCullItems; ++k) {
      const u32 id = p * kCullTile + k * kCullThreads + tid;
      px[k] = py[k] = pz[k] = 0.0f;
      visbits[k] = 0;
      if (id < n) {
        px[k] = __ldg(a.position + 3 * (size_t)id + 0);
        py[k] = __ldg(a.position + 3 * (size_t)id + 1);
        pz[k] = __ldg(a.position + 3 * (size_t)id + 2);
      }
    }
#pragma unroll 1
    for (u32 v = 0; v < nv; ++v) {
#pragma unroll
      for (u32 k = 0; k < kCullItems; ++k) {
        bool vis = false;
        if (p * kCullTile + k * kCullThreads + tid < n) {
          const float q[4] = {px[k], py[k], pz[k], 1.0f};
          float c[4];
          mat4_vec4(a.fc[v].pvm, q, c);
          const float x = c[0] / c[3], y = c[1] / c[3], z = c[2] / c[3];
          vis = fabsf(x) <= 1.0f && fabsf(y) <= 1.0f && z >= 0.0f && z <= 1.0f;
        }
        visbits[k] |= (vis ? 1u : 0u) << v;
        const u32 ball = __ballot_sync(0xffffffffu, vis);
        if (lane == 0) s_cnt[v][k][warp] = __popc(ball);
      }
    }
    __syncthreads();
    if (tid < nv) {  // view tid: offsets of its warps; its aggregate is published now, resolved later
      u32 acc = 0;
      for (u32 k = 0; k < kCullItems; ++k)
        for (u32 w = 0; w < kCullThreads / 32; ++w) {
          const u32 c = s_cnt[tid][k][w];
          s_cnt[tid][k][w] = acc;
          acc += c;
        }
      s_acc[tid] = acc;
      lb_publish(a.view[tid].status, 1, p, a.epoch, acc);
    }
    // project every visible (splat, view) -- records are written by id and need no offset
#pragma unroll 1
    for (u32 k = 0; k < kCullItems; ++k) {
      const u32 id = p * kCullTile + k * kCullThreads + tid;
#pragma unroll 1
      for (u32 v = 0; v < nv; ++v) {  // the same view across the warp: no divergence between views
        if ((visbits[k] >> v) & 1u) {
          ca.record = a.view[v].record;
          project_splat<SH32>(a.fc[v], ca, id, px[k], py[k], pz[k]);
        }
      }
    }
    if (tid < nv) {
      const u32 acc = s_acc[tid];
      const u32 excl = lb_resolve(a.view[tid].status, 1, p, a.epoch, acc, a.err);
      s_base[tid] = excl;
      if (p == nparts - 1) *a.view[tid].visible_count = excl + acc;
    }
    __syncthreads();
#pragma unroll 1
    for (u32 k = 0; k < kCullItems; ++k) {
      const u32 id = p * kCullTile + k * kCullThreads + tid;
#pragma unroll 1
      for (u32 v = 0; v < nv; ++v) {
        const bool vis = (visbits[k] >> v) & 1u;
        const u32 ball = __ballot_sync(0xffffffffu, vis);
        if (vis) {
          const float q[4] = {px[k], py[k], pz[k], 1.0f};
          float c[4];
          mat4_vec4(a.fc[v].pvm, q, c);
          const u32 slot = s_base[v] + s_cnt[v][k][warp] + __popc(ball & lt);
          a.view[v].key[slot] = __float_as_uint(1.0f - c[2] / c[3]);
          a.view[v].index[slot] = id;
        }
      }
    }
    __syncthreads();
  }
}

cudaError_t launch_cull_views(const CullViewsArgs& a, cudaStream_t stream) {
  if (a.n == 0 || a.count == 0) return cudaSuccess;
  if (a.count > kMaxCullViews) return cudaErrorInvalidValue;
  const u32 parts = (a.n + kCullTile - 1) / kCullTile;
  const int sms = a.num_sms > 0 ? a.num_sms : 1;
  if (a.sh32)
    k_cull_views<true><<<min(parts, (u32)sms * 8u), kCullThreads, 0, stream>>>(a);
  else
    k_cull_views<false><<<min(parts, (u32)sms * 8u), kCullThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

const void* cull_project_kernel() { return reinterpret_cast<const void*>(&k_cull_project<false>); }

cudaError_t launch_cull_project(const FrameConst& fc, const CullArgs& a, cudaStream_t stream) {
  if (fc.n == 0) return cudaSuccess;
  const u32 parts = (fc.n + kCullTile - 1) / kCullTile;
  const int sms = a.num_sms > 0 ? a.num_sms : 1;
  const u32 grid = min(parts, (u32)sms * 8u);
  if (a.sh32)
    k_cull_project<true><<<grid, kCullThreads, 0, stream>>>(fc, a);
  else
    k_cull_project<false><<<grid, kCullThreads, 0, stream>>>(fc, a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Instance records in sorted order + indirect draw arguments (projection.comp:64-75, 177-179).

__global__ void k_instances(const u32* __restrict__ index, const u32* __restrict__ visible_count,
                            const float4* __restrict__ inst_by_id, u32 n, float4* __restrict__ instances,
                            u32* __restrict__ draw) {
  const u32 v = min(*visible_count, n);
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 r = blockIdx.x * blockDim.x + threadIdx.x; instances && r < v; r += stride) {
    const u32 id = index[r];
    instances[3 * (size_t)r + 0] = inst_by_id[3 * (size_t)id + 0];
    instances[3 * (size_t)r + 1] = inst_by_id[3 * (size_t)id + 1];
    instances[3 * (size_t)r + 2] = inst_by_id[3 * (size_t)id + 2];
  }
  if (draw && blockIdx.x == 0 && threadIdx.x == 0) {
    draw[0] = 6 * v;  // indexCount
    draw[1] = 1;      // instanceCount
    draw[2] = 0;      // firstIndex
    draw[3] = 0;      // vertexOffset
    draw[4] = 0;      // firstInstance
    draw[5] = draw[6] = draw[7] = 0;
    draw[8] = v;      // vertexCount of the point-list draw
    draw[9] = 1;
    draw[10] = 0;
    draw[11] = 0;
  }
}

cudaError_t launch_instances(const u32* index, const u32* visible_count, const float* inst_by_id, u32 n,
                             float* instances, u32* draw_indirect, cudaStream_t stream) {
  const u32 grid = max(1u, min((n + 255) / 256, 4096u));
  k_instances<<<grid, 256, 0, stream>>>(index, visible_count, reinterpret_cast<const float4*>(inst_by_id), n,
                                        reinterpret_cast<float4*>(instances), draw_indirect);
  return cudaGetLastError();
}

}  // namespace gs
