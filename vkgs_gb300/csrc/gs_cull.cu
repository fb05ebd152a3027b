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

// The projection of one visible splat from its values: c0..c5 = cov3d, shv = its 48 binary16 SH as
// 6 x 16 bytes (global memory, or shared memory with SMEM), o = opacity.  SH32: FP32 coefficients read
// from a.sh32 instead (the differentiable path) -- a separate instantiation, so the plain path keeps
// its register count.
template <bool SH32, bool SMEM = false>
__device__ __forceinline__ void project_values(const FrameConst& fc, const CullArgs& a, u32 id, float x0, float y0,
                                               float z0, float c0, float c1, float c2, float c3, float c4, float c5,
                                               const uint4* shv, float o);

template <bool SH32>
__device__ void project_splat(const FrameConst& fc, const CullArgs& a, u32 id, float x0, float y0, float z0) {
  const float* cv = a.cov3d + 6 * (size_t)id;
  project_values<SH32>(fc, a, id, x0, y0, z0, __ldg(cv + 0), __ldg(cv + 1), __ldg(cv + 2), __ldg(cv + 3),
                       __ldg(cv + 4), __ldg(cv + 5), reinterpret_cast<const uint4*>(a.sh + 48 * (size_t)id),
                       __ldg(a.opacity + id));
}

template <bool SH32, bool SMEM>
__device__ __forceinline__ void project_values(const FrameConst& fc, const CullArgs& a, u32 id, float x0, float y0,
                                               float z0, float c0, float c1, float c2, float c3, float c4, float c5,
                                               const uint4* shv, float o) {
  // direction for SH in model space (projection.comp:85-87); normalize = v / sqrt(dot(v, v))
  const float ddx = x0 - fc.cam_m[0], ddy = y0 - fc.cam_m[1], ddz = z0 - fc.cam_m[2];
  const float dl = sqrtf((ddx * ddx + ddy * ddy) + ddz * ddz);
  const float x = ddx / dl, y = ddy / dl, z = ddz / dl;

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
      unpack_half8(SMEM ? shv[2 * ch] : __ldg(shv + 2 * ch), g);
      unpack_half8(SMEM ? shv[2 * ch + 1] : __ldg(shv + 2 * ch + 1), g + 8);
    }
    const float col = ((dot4(b00, b01, b02, b03, g[0], g[1], g[2], g[3]) +
                        dot4(b10, b11, b12, b13, g[4], g[5], g[6], g[7])) +
                       dot4(b20, b21, b22, b23, g[8], g[9], g[10], g[11])) +
                      dot4(b30, b31, b32, b33, g[12], g[13], g[14], g[15]);
    color[ch] = fmaxf(col + 0.5f, 0.0f);
  }

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

// ---------------------------------------------------------------------------------------------
// The same pass with the splat buffers streamed into shared memory by the Tensor Memory Accelerator.
// Partitions of kStreamSplats splats (one per compute thread); each CTA keeps two partitions in
// flight: while it culls, projects and compacts one, the bulk copies (cp.async.bulk, completion counted
// in bytes on an mbarrier) of the next land in the other stage.  The copies move every byte of the
// partition's position, cov3d, opacity and SH rows -- also those of splats that turn out invisible,
// whose sectors DRAM delivers anyway when the per-thread loads skip them -- so the scene streams at the
// copy engine's rate with no registers held for loads in flight.  Arithmetic and outputs are those of
// k_cull_project (the same device functions), bit for bit.  The last partition, when partial, is
// loaded by the threads (its byte counts need not be multiples of 16).
//
// Warp specialisation: eight compute warps and a control warp.  The control warp takes the tickets,
// arms and issues the bulk copies, publishes each partition's count and resolves the look-back of the
// PREVIOUS partition while the compute warps project the current one; the compute warps write a
// partition's keys and ids one iteration later, once its offset is known.  Nothing on the compute
// warps' path waits for another CTA.
constexpr u32 kStreamSplats = 256;
constexpr u32 kStreamThreads = kStreamSplats + 32;
struct StreamStage {
  float pos[kStreamSplats * 3];
  float cov[kStreamSplats * 6];
  float opa[kStreamSplats];
  uint4 sh[kStreamSplats * 6];
};
constexpr u32 kStageBytes = (u32)sizeof(StreamStage);
static_assert(kStageBytes == kStreamSplats * (12 + 24 + 4 + 96), "stage layout");
static_assert(kStreamSplats == kCullStatusSplats, "one look-back status word per partition");
constexpr u32 kStreamSmem = 2 * kStageBytes;
// resident CTAs per SM the grid is sized for (at most 3 fit the shared memory)
#ifndef GS_STREAM_CTAS_PER_SM
#define GS_STREAM_CTAS_PER_SM 3
#endif
constexpr u32 kStreamCtasPerSm = GS_STREAM_CTAS_PER_SM;

__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, u32 bytes, u64* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Waits (bounded) for phase `parity` of the barrier; false when the wait gave up.
__device__ __forceinline__ bool mbar_wait(u64* bar, u32 parity) {
  for (u32 spin = 0; spin < kMaxSpins; ++spin) {
    u32 done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void compute_bar() {  // the compute warps only (named barrier 1)
  asm volatile("bar.sync 1, %0;" ::"n"(kStreamSplats) : "memory");
}

__global__ __launch_bounds__(kStreamThreads, 3) void k_cull_stream(const FrameConst fc, const CullArgs a) {
  extern __shared__ __align__(128) unsigned char s_dyn[];
  StreamStage* stage = reinterpret_cast<StreamStage*>(s_dyn);
  constexpr u32 kW = kStreamSplats / 32;  // compute warps
  __shared__ u64 s_bar[2];
  __shared__ u32 s_ticket[2];
  __shared__ u32 s_cnt[2][kW], s_off[2][kW];
  __shared__ u32 s_key[2][kStreamSplats];
  __shared__ u32 s_acc[2], s_base[2], s_abort;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const bool control = warp == kW;
  const u32 n = fc.n;
  const u32 nparts = (n + kStreamSplats - 1) / kStreamSplats;
  const bool partial_tail = (n % kStreamSplats) != 0;

  // control lane 0: the four bulk copies of partition p into stage s (none for a partial last partition)
  const auto issue = [&](u32 s, u32 p) {
    if (p >= nparts || (partial_tail && p == nparts - 1)) return;
    const size_t b = (size_t)p * kStreamSplats;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage's earlier reads come first
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&s_bar[s])),
                 "r"(kStageBytes)
                 : "memory");
    bulk_copy_g2s(stage[s].pos, a.position + 3 * b, kStreamSplats * 12, &s_bar[s]);
    bulk_copy_g2s(stage[s].cov, a.cov3d + 6 * b, kStreamSplats * 24, &s_bar[s]);
    bulk_copy_g2s(stage[s].opa, a.opacity + b, kStreamSplats * 4, &s_bar[s]);
    bulk_copy_g2s(stage[s].sh, a.sh + 48 * b, kStreamSplats * 96, &s_bar[s]);
  };
  // the control warp: the offset of partition q (stage qs) from the look-back
  const auto resolve = [&](u32 q, u32 qs) {
    const u32 acc = s_acc[qs];
    const u32 excl = lb_resolve_warp(a.status, 1, q, a.epoch, acc, a.err);
    if (lane == 0) {
      s_base[qs] = excl;
      if (q == nparts - 1) *a.visible_count = excl + acc;
    }
  };
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_abort = 0;
    s_ticket[0] = atomicAdd(a.ticket, 1u);
    s_ticket[1] = atomicAdd(a.ticket, 1u);
    issue(0, s_ticket[0]);
    issue(1, s_ticket[1]);
  }
  __syncthreads();
  u32 parity = 0;  // bit s: the phase stage s waits for next
  const u32 ltm = lanemask_lt();
  bool have_prev = false, vis_prev = false;
  u32 q = 0, ball_prev = 0, s = 0;
  for (;; s ^= 1u) {
    const u32 p = s_ticket[s];
    if (p >= nparts) break;
    const u32 base = p * kStreamSplats;
    const bool tail = partial_tail && p == nparts - 1;
    StreamStage& st = stage[s];
    bool vis = false;
    u32 ball = 0;
    float x = 0.0f, y = 0.0f, z = 0.0f;
    if (!control) {
      if (tail) {
        const u32 cnt = n - base;
        for (u32 i = tid; i < 3 * cnt; i += kStreamSplats) st.pos[i] = __ldg(a.position + 3 * (size_t)base + i);
        for (u32 i = tid; i < 6 * cnt; i += kStreamSplats) st.cov[i] = __ldg(a.cov3d + 6 * (size_t)base + i);
        for (u32 i = tid; i < cnt; i += kStreamSplats) st.opa[i] = __ldg(a.opacity + base + i);
        const uint4* shg = reinterpret_cast<const uint4*>(a.sh + 48 * (size_t)base);
        for (u32 i = tid; i < 6 * cnt; i += kStreamSplats) st.sh[i] = __ldg(shg + i);
        compute_bar();
      } else if (!mbar_wait(&s_bar[s], (parity >> s) & 1u)) {
        atomicOr(&s_abort, 1u);
      }
      const u32 id = base + tid;
      if (id < n) {
        x = st.pos[3 * tid + 0];
        y = st.pos[3 * tid + 1];
        z = st.pos[3 * tid + 2];
        const float v[4] = {x, y, z, 1.0f};
        float c[4];
        mat4_vec4(fc.pvm, v, c);
        const float cx = c[0] / c[3], cy = c[1] / c[3], cz = c[2] / c[3];
        vis = fabsf(cx) <= 1.0f && fabsf(cy) <= 1.0f && cz >= 0.0f && cz <= 1.0f;
        s_key[s][tid] = __float_as_uint(1.0f - cz);
      }
      ball = __ballot_sync(0xffffffffu, vis);
      if (lane == 0) s_cnt[s][warp] = __popc(ball);
    }
    if (!tail) parity ^= 1u << s;
    __syncthreads();  // A: the partition is culled
    if (s_abort) {  // a stage's copies never completed: record it, give the copies in flight a last
                    // bounded wait, and leave
      if (tid == 0) {
        atomicOr(a.err, ERR_TIMEOUT);
        mbar_wait(&s_bar[s], ((parity >> s) & 1u) ^ 1u);
        const u32 other = s_ticket[s ^ 1u];
        if (other < nparts && !(partial_tail && other == nparts - 1))
          mbar_wait(&s_bar[s ^ 1u], (parity >> (s ^ 1u)) & 1u);
      }
      return;
    }
    if (control) {
      if (lane == 0) {  // publish this partition's count at once
        u32 acc = 0;
        for (u32 w = 0; w < kW; ++w) {
          s_off[s][w] = acc;
          acc += s_cnt[s][w];
        }
        s_acc[s] = acc;
        lb_publish(a.status, 1, p, a.epoch, acc);
      }
      __syncwarp();
      if (have_prev) resolve(q, s ^ 1u);  // overlaps the projection below
    } else if (vis) {
      const float* cv = st.cov + 6 * tid;
      project_values<false, true>(fc, a, base + tid, x, y, z, cv[0], cv[1], cv[2], cv[3], cv[4], cv[5],
                                  st.sh + 6 * tid, st.opa[tid]);
    }
    __syncthreads();  // B: the stage is read and the previous partition's offset is known
    if (control) {
      if (lane == 0) {
        const u32 next = atomicAdd(a.ticket, 1u);
        s_ticket[s] = next;
        issue(s, next);
      }
    } else if (have_prev && vis_prev) {
      const u32 qs = s ^ 1u;
      const u32 slot = s_base[qs] + s_off[qs][warp] + __popc(ball_prev & ltm);
      a.key[slot] = s_key[qs][tid];
      a.index[slot] = q * kStreamSplats + tid;
    }
    have_prev = true;
    q = p;
    vis_prev = vis;
    ball_prev = ball;
  }
  if (!have_prev) return;
  if (control) resolve(q, s ^ 1u);  // the last partition of this CTA
  __syncthreads();
  if (!control && vis_prev) {
    const u32 qs = s ^ 1u;
    const u32 slot = s_base[qs] + s_off[qs][warp] + __popc(ball_prev & ltm);
    a.key[slot] = s_key[qs][tid];
    a.index[slot] = q * kStreamSplats + tid;
  }
}

bool cull_stream_usable(const CullArgs& a) {
  const auto aligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  return !a.sh32 && aligned(a.position) && aligned(a.cov3d) && aligned(a.opacity) && aligned(a.sh);
}

cudaError_t cull_stream_init() {
  return cudaFuncSetAttribute(k_cull_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStreamSmem);
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

bool is_cull_kernel(const void* f) {
  return f == reinterpret_cast<const void*>(&k_cull_project<false>) || f == reinterpret_cast<const void*>(&k_cull_stream);
}

cudaError_t launch_cull_project(const FrameConst& fc, const CullArgs& a, cudaStream_t stream) {
  if (fc.n == 0) return cudaSuccess;
  const int sms = a.num_sms > 0 ? a.num_sms : 1;
  if (a.staged && cull_stream_usable(a)) {
    const u32 parts = (fc.n + kStreamSplats - 1) / kStreamSplats;
    k_cull_stream<<<min(parts, (u32)sms * kStreamCtasPerSm), kStreamThreads, kStreamSmem, stream>>>(fc, a);
    return cudaGetLastError();
  }
  const u32 parts = (fc.n + kCullTile - 1) / kCullTile;
  const u32 grid = min(parts, (u32)sms * (a.lean ? kLeanCullCtasPerSm : kCullCtasPerSm));
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
