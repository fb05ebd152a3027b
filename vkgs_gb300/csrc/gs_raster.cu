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
// the restatement's.  Each warp owns an 8x4 pixel block and walks only the records whose quad can
// reach that block (a conservative per-batch test), which leaves every pixel's sum unchanged.  Each
// pixel stops blending exactly when its transmittance falls below t_floor (the splats behind can then
// change no channel by more than t_floor), so its sum does not depend on how pixels are grouped into
// warps; a warp stops walking once all its pixels have stopped, and the tile once all its warps have.  The sorted splats arrive in depth
// slabs, nearest first: a tile that is not finished stores its pixels' running sums for the next
// slab's launch, a finished one writes its pixels and is marked done (later slabs skip it), and the
// last slab writes every remaining tile.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

constexpr int kRasterThreads = kTile * kTile;  // one pixel per thread
constexpr int kWarps = kRasterThreads / 32;
constexpr int kBlockW = 8, kBlockH = 4;            // each warp owns an 8x4 pixel block of the tile
constexpr int kBlocksX = kTile / kBlockW;          // 2 x 4 blocks
static_assert(kBlockW * kBlockH == 32 && (kTile / kBlockW) * (kTile / kBlockH) == kWarps, "warp blocks");

// Blocks of the tile (bit b = block (b % 2, b / 2)) that the quad of one record may touch: the
// separating-axis test of two rectangles -- the block's rectangle of pixel centres against the quad,
// on the block axes (the quad's axis-aligned extent from its rot_scale columns, widened by the same
// 0.25-pixel margin the tile binning uses) and on the quad's own axes u and v (the rows of
// rot_scale^-1 the blend evaluates, widened by a rounding margin far above the error of either
// evaluation).  A cleared bit therefore means no pixel centre of the block is covered, and the
// record changes none of its pixels.
template <int BW = kBlockW, int BH = kBlockH>
__device__ __forceinline__ u32 block_mask(const float4 q0, const float4 q1, const float4 q3, float ox, float oy,
                                          float sx, float sy, float mx, float my) {
  // ox, oy: NDC of the tile's first pixel centre; sx, sy: NDC step between pixel centres
  constexpr int kBX = kTile / BW;
  const float hx = 0.5f * (BW - 1) * sx, hy = 0.5f * (BH - 1) * sy;  // block half extents
  const float ex = 3.0f * (fabsf(q3.x) + fabsf(q3.z)) + mx + hx;
  const float ey = 3.0f * (fabsf(q3.y) + fabsf(q3.w)) + my + hy;
  const float au0 = fabsf(q0.z), au1 = fabsf(q0.w), av0 = fabsf(q1.x), av1 = fabsf(q1.y);
  const float ru = au0 * hx + au1 * hy, rv = av0 * hx + av1 * hy;
  u32 m = 0;
#pragma unroll
  for (int by = 0; by < kTile / BH; ++by) {
    const float dy = oy + (by * BH + 0.5f * (BH - 1)) * sy - q0.y;
#pragma unroll
    for (int bx = 0; bx < kBX; ++bx) {
      const float dx = ox + (bx * BW + 0.5f * (BW - 1)) * sx - q0.x;
      const float u = q0.z * dx + q0.w * dy, v = q1.x * dx + q1.y * dy;
      const float tu = 3.0f + ru + 4e-6f * (au0 * (fabsf(dx) + hx) + au1 * (fabsf(dy) + hy)) + 1e-3f;
      const float tv = 3.0f + rv + 4e-6f * (av0 * (fabsf(dx) + hx) + av1 * (fabsf(dy) + hy)) + 1e-3f;
      const bool hit = fabsf(dx) <= ex && fabsf(dy) <= ey && fabsf(u) <= tu && fabsf(v) <= tv;
      m |= hit ? 1u << (by * kBX + bx) : 0u;
    }
  }
  return m;
}

// TRAIN (the differentiable forward): every pixel also records how many list entries it blended
// (nproc) and its final transmittance, which is all the backward needs to walk the list in reverse.
// COUNT blends every fragment (no stop) and counts the covered ones.
template <bool DEPTH, bool COUNT, bool TRAIN>
__global__ __launch_bounds__(kRasterThreads, 5) void k_raster(const RasterArgs a) {
  __shared__ float4 s_q0[kRasterThreads];  // cx, cy, m00, m01
  __shared__ float4 s_q1[kRasterThreads];  // m10, m11, cz, opacity
  __shared__ float4 s_q2[kRasterThreads];  // r, g, b, -
  __shared__ u32 s_bits[kWarps][kWarps];   // [block][32-record word]: records that may touch the block
  const u32 tile = blockIdx.x;
  if (!a.first && ((a.tile_done[tile >> 5] >> (tile & 31u)) & 1u)) return;  // finished by an earlier slab
  const u32 tx = tile % a.tiles_x, ty = tile / a.tiles_x;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 px = tx * kTile + (warp % kBlocksX) * kBlockW + lane % kBlockW;
  const u32 py = ty * kTile + (warp / kBlocksX) * kBlockH + lane / kBlockW;
  const bool inside = px < a.width && py < a.height;
  const float fx = __fdiv_rn((float)(2 * px + 1), (float)a.width) - 1.0f;
  const float fy = __fdiv_rn((float)(2 * py + 1), (float)a.height) - 1.0f;
  const float dpix = (DEPTH && inside) ? a.depth[(size_t)py * a.width + px] : 1.0f;
  const uint2 tr = reinterpret_cast<const uint2*>(a.tile_range)[tile];
  const uint2 range = make_uint2(min(tr.x, a.pair_capacity), min(tr.y, a.pair_capacity));
  // tile geometry for the block test
  const float sx = 2.0f / (float)a.width, sy = 2.0f / (float)a.height;
  const float ox = (float)(2 * tx * kTile + 1) / (float)a.width - 1.0f;
  const float oy = (float)(2 * ty * kTile + 1) / (float)a.height - 1.0f;
  const float mx = 0.5f * sx, my = 0.5f * sy;  // 0.25 pixel

  const size_t pix = (size_t)py * a.width + px;
  float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f, ca = 0.0f;
  if (!a.first && inside) {  // the running sums of the nearer slabs
    const float4 c = a.state_c[pix];
    cr = c.x, cg = c.y, cb = c.z, ca = c.w;
    T = a.state_t[pix];
  }
  u32 frags = 0, needed = 0, blended = 0;
  const float kExp = -0.5f * 1.4426950408889634f;  // -log2(e)/2
  bool done = !inside || (!COUNT && T < a.t_floor);
  for (u32 hi = range.y; hi > range.x;) {
    const u32 lo = (hi - range.x > (u32)kRasterThreads) ? hi - kRasterThreads : range.x;
    const u32 cnt = hi - lo;
    u32 mask = 0;
    if (tid < cnt) {
      const u32 id = a.pair_splat[hi - 1 - tid];  // nearest first
      const float4* rec = a.record + 4 * (size_t)id;
      const float4 q0 = rec[REC_CENTER], q1 = rec[REC_ROW1], q3 = rec[REC_AXES];
      s_q0[tid] = q0;
      s_q1[tid] = q1;
      s_q2[tid] = rec[REC_COLOR];
      mask = block_mask(q0, q1, q3, ox, oy, sx, sy, mx, my);
    }
#pragma unroll
    for (int b = 0; b < kWarps; ++b) {
      const u32 bits = __ballot_sync(0xffffffffu, (mask >> b) & 1u);
      if (lane == 0) s_bits[b][warp] = bits;
    }
    __syncthreads();
    if (!__all_sync(0xffffffffu, done)) {
      for (int k = 0; k < kWarps; ++k) {
        u32 word = s_bits[warp][k];
        while (word) {
          const u32 j = 32u * k + (u32)(__ffs(word) - 1);
          word &= word - 1u;
          const float4 q0 = s_q0[j], q1 = s_q1[j];
          const float dx = __fsub_rn(fx, q0.x), dy = __fsub_rn(fy, q0.y);
          const float u = __fadd_rn(__fmul_rn(q0.z, dx), __fmul_rn(q0.w, dy));
          const float v = __fadd_rn(__fmul_rn(q1.x, dx), __fmul_rn(q1.y, dy));
          bool cov = (fabsf(u) <= 3.0f) & (fabsf(v) <= 3.0f);
          if (DEPTH) cov &= q1.z < dpix;
          if (COUNT) {
            frags += (cov && inside) ? 1u : 0u;
            needed += (cov && inside && T >= a.t_floor) ? 1u : 0u;
          } else {
            cov &= T >= a.t_floor;  // a pixel stops exactly when its transmittance falls below t_floor
          }
          const float g = cov ? exp2f(__fmul_rn(__fmaf_rn(u, u, __fmul_rn(v, v)), kExp)) : 0.0f;
          const float al = __fmul_rn(q1.w, g);
          const float w = al * T;
          const float4 q2 = s_q2[j];
          cr += w * q2.x;
          cg += w * q2.y;
          cb += w * q2.z;
          ca += w * al;
          T -= w;
          if (TRAIN && cov) blended = range.y - hi + j + 1;  // processing index + 1 (0 = nearest)
        }
        // A warp whose 32 pixels are all below t_floor stops here (the remaining records can move no
        // channel of these pixels by more than t_floor).
        if (!COUNT && __all_sync(0xffffffffu, done || T < a.t_floor)) break;
      }
    }
    hi = lo;
    if (!COUNT) done = done || T < a.t_floor;
    // Barrier before the next batch overwrites shared memory; also ends the tile once all are done.
    if (__syncthreads_and(done)) break;
  }
  // Finished: every pixel below t_floor (never while counting, which disables the early stop).
  const bool finished = __syncthreads_and(done);
  if (finished && !a.last && tid == 0) atomicOr(a.tile_done + (tile >> 5), 1u << (tile & 31u));
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      frags += __shfl_xor_sync(0xffffffffu, frags, o);
      needed += __shfl_xor_sync(0xffffffffu, needed, o);
    }
    if (lane == 0 && frags) atomicAdd(a.fragments, (unsigned long long)frags);
    if (lane == 0 && needed) atomicAdd(a.fragments + 1, (unsigned long long)needed);
  }
  if (!inside) return;
  if (TRAIN) {
    a.nproc[pix] = blended;
    a.state_t[pix] = T;
  }
  if (!finished && !a.last) {  // a farther slab continues these pixels
    a.state_c[pix] = make_float4(cr, cg, cb, ca);
    a.state_t[pix] = T;
    return;
  }
  const float alpha = ca + T;
  if (a.out_rgba) reinterpret_cast<float4*>(a.out_rgba)[pix] = make_float4(cr, cg, cb, alpha);
  if (a.out_bgra) {
    const auto q = [](float x) { return (unsigned char)__float2uint_rn(__saturatef(x) * 255.0f); };
    a.out_bgra[pix] = make_uchar4(q(cb), q(cg), q(cr), q(alpha));
  }
}

// The plain, counting and differentiable forwards with two horizontally adjacent pixels per thread: 128 threads
// per tile, each warp owning an 8x8 block (4 pixel pairs x 8 rows).  A record's shared-memory loads,
// the walk over the block's record bits and the vertical offset serve both pixels of a thread; each
// pixel's coverage test keeps the explicitly rounded scalar operations above (the pair's dx is one
// packed add of the negated centre, exact), so the covered set is still exactly the restatement's,
// and the Gaussian and the blend run as packed FP32 pairs, one instruction for both pixels.  Shared
// memory holds the values the packed operations take twice, side by side.
constexpr int kPairThreads = kTile * kTile / 2;
constexpr int kPairWarps = kPairThreads / 32;  // 4 blocks of 64 pixels
constexpr int kPairBatch = 128;                // records per batch, one per thread (256: ~1 % fewer frames/s in flight)
constexpr int kPairLoads = kPairBatch / kPairThreads;
constexpr int kPairWords = kPairBatch / 32;
static_assert(kPairLoads >= 1 && kPairBatch % kPairThreads == 0, "every thread loads whole records");

constexpr int kPairBW = 8, kPairBH = 8, kPairBX = kTile / kPairBW;  // 8x8 blocks, 2 x 2 per tile
static_assert(kPairWarps * kPairBW * kPairBH == kTile * kTile && kPairBW * kPairBH == 64, "pair blocks");

// 9 CTAs per SM (56 registers): 921-922 vs 918 frames/s with frames in flight against 8 (64 registers)
template <bool DEPTH, bool COUNT, bool TRAIN>
__global__ __launch_bounds__(kPairThreads, 9) void k_raster_pairs(const RasterArgs a) {
  __shared__ float4 s_a[kPairBatch];  // (-cx, -cx, -cy, m00)
  __shared__ float4 s_b[kPairBatch];  // (m01, m10, m11, z)
  __shared__ float4 s_c[kPairBatch];  // (r, r, g, g)
  __shared__ float4 s_d[kPairBatch];  // (b, b, opacity, opacity)
  __shared__ u32 s_bits[kPairWarps][kPairWords];  // [block][32-record word]
  const u32 tile = blockIdx.x;
  if (!a.first && ((a.tile_done[tile >> 5] >> (tile & 31u)) & 1u)) return;  // finished by an earlier slab
  const u32 tx = tile % a.tiles_x, ty = tile / a.tiles_x;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 px = tx * kTile + (warp % kPairBX) * kPairBW + 2 * (lane % (kPairBW / 2));  // pair (px, px + 1)
  const u32 py = ty * kTile + (warp / kPairBX) * kPairBH + lane / (kPairBW / 2);
  const bool in0 = px < a.width && py < a.height, in1 = px + 1 < a.width && py < a.height;
  const float2 fx = make_float2(__fdiv_rn((float)(2 * px + 1), (float)a.width) - 1.0f,
                                __fdiv_rn((float)(2 * px + 3), (float)a.width) - 1.0f);
  const float fy = __fdiv_rn((float)(2 * py + 1), (float)a.height) - 1.0f;
  const size_t pix = (size_t)py * a.width + px;
  float2 dpix = make_float2(1.0f, 1.0f);
  if (DEPTH) {
    if (in0) dpix.x = a.depth[pix];
    if (in1) dpix.y = a.depth[pix + 1];
  }
  const uint2 tr = reinterpret_cast<const uint2*>(a.tile_range)[tile];
  const uint2 range = make_uint2(min(tr.x, a.pair_capacity), min(tr.y, a.pair_capacity));
  const float sx = 2.0f / (float)a.width, sy = 2.0f / (float)a.height;
  const float ox = (float)(2 * tx * kTile + 1) / (float)a.width - 1.0f;
  const float oy = (float)(2 * ty * kTile + 1) / (float)a.height - 1.0f;
  const float mx = 0.5f * sx, my = 0.5f * sy;  // 0.25 pixel

  float2 T = make_float2(1.0f, 1.0f), cr = make_float2(0.0f, 0.0f), cg = cr, cb = cr, ca = cr;
  if (!a.first) {  // the running sums of the nearer slabs
    if (in0) {
      const float4 c = a.state_c[pix];
      cr.x = c.x, cg.x = c.y, cb.x = c.z, ca.x = c.w;
      T.x = a.state_t[pix];
    }
    if (in1) {
      const float4 c = a.state_c[pix + 1];
      cr.y = c.x, cg.y = c.y, cb.y = c.z, ca.y = c.w;
      T.y = a.state_t[pix + 1];
    }
  }
  u32 frags = 0, needed = 0, blended0 = 0, blended1 = 0;
  const float kExp = -0.5f * 1.4426950408889634f;  // -log2(e)/2
  const float2 kExp2 = make_float2(kExp, kExp), kMinus1 = make_float2(-1.0f, -1.0f);
  const auto stopped = [&]() {
    return (!in0 || (!COUNT && T.x < a.t_floor)) && (!in1 || (!COUNT && T.y < a.t_floor));
  };
  bool done = stopped();
  for (u32 hi = range.y; hi > range.x;) {
    const u32 lo = (hi - range.x > (u32)kPairBatch) ? hi - kPairBatch : range.x;
    const u32 cnt = hi - lo;
#pragma unroll
    for (int r = 0; r < kPairLoads; ++r) {
      const u32 j = tid + r * kPairThreads;
      u32 m = 0;
      if (j < cnt) {
        const u32 id = a.pair_splat[hi - 1 - j];  // nearest first
        const float4* rec = a.record + 4 * (size_t)id;
        const float4 q0 = rec[REC_CENTER], q1 = rec[REC_ROW1], q3 = rec[REC_AXES], q2 = rec[REC_COLOR];
        s_a[j] = make_float4(-q0.x, -q0.x, -q0.y, q0.z);
        s_b[j] = make_float4(q0.w, q1.x, q1.y, q1.z);
        s_c[j] = make_float4(q2.x, q2.x, q2.y, q2.y);
        s_d[j] = make_float4(q2.z, q2.z, q1.w, q1.w);
        m = block_mask<kPairBW, kPairBH>(q0, q1, q3, ox, oy, sx, sy, mx, my);
      }
#pragma unroll
      for (int b = 0; b < kPairWarps; ++b) {
        const u32 bits = __ballot_sync(0xffffffffu, (m >> b) & 1u);
        if (lane == 0) s_bits[b][r * kPairWarps + warp] = bits;
      }
    }
    __syncthreads();
    if (!__all_sync(0xffffffffu, done)) {
      for (int k = 0; k < kPairWords; ++k) {
        u32 word = s_bits[warp][k];
        while (word) {
          const u32 j = 32u * k + (u32)(__ffs(word) - 1);
          word &= word - 1u;
          const float4 A = s_a[j], B = s_b[j];
          const float2 dx = __fadd2_rn(fx, make_float2(A.x, A.y));  // fx - cx for both pixels
          const float dy = __fadd_rn(fy, A.z);
          const float wu = __fmul_rn(B.x, dy), wv = __fmul_rn(B.z, dy);
          const float u0 = __fadd_rn(__fmul_rn(A.w, dx.x), wu), u1 = __fadd_rn(__fmul_rn(A.w, dx.y), wu);
          const float v0 = __fadd_rn(__fmul_rn(B.y, dx.x), wv), v1 = __fadd_rn(__fmul_rn(B.y, dx.y), wv);
          bool c0 = (fabsf(u0) <= 3.0f) & (fabsf(v0) <= 3.0f);
          bool c1 = (fabsf(u1) <= 3.0f) & (fabsf(v1) <= 3.0f);
          if (DEPTH) {
            c0 &= B.w < dpix.x;
            c1 &= B.w < dpix.y;
          }
          if (COUNT) {
            frags += ((c0 && in0) ? 1u : 0u) + ((c1 && in1) ? 1u : 0u);
            needed += ((c0 && in0 && T.x >= a.t_floor) ? 1u : 0u) + ((c1 && in1 && T.y >= a.t_floor) ? 1u : 0u);
          } else {
            c0 &= T.x >= a.t_floor;
            c1 &= T.y >= a.t_floor;
          }
          if (TRAIN) {  // processing index + 1 (0 = nearest)
            if (c0) blended0 = range.y - hi + j + 1;
            if (c1) blended1 = range.y - hi + j + 1;
          }
          const float2 uu = make_float2(u0, u1), vv = make_float2(v0, v1);
          const float2 e = __fmul2_rn(__ffma2_rn(uu, uu, __fmul2_rn(vv, vv)), kExp2);
          const float2 g = make_float2(c0 ? exp2f(e.x) : 0.0f, c1 ? exp2f(e.y) : 0.0f);
          const float4 C = s_c[j], D = s_d[j];
          const float2 al = __fmul2_rn(make_float2(D.z, D.w), g);
          const float2 w = __fmul2_rn(al, T);
          cr = __ffma2_rn(w, make_float2(C.x, C.y), cr);
          cg = __ffma2_rn(w, make_float2(C.z, C.w), cg);
          cb = __ffma2_rn(w, make_float2(D.x, D.y), cb);
          ca = __ffma2_rn(w, al, ca);
          T = __ffma2_rn(w, kMinus1, T);
        }
        // A warp whose 64 pixels are all below t_floor stops here.
        if (!COUNT && __all_sync(0xffffffffu, stopped())) break;
      }
    }
    hi = lo;
    done = done || stopped();
    // Barrier before the next batch overwrites shared memory; also ends the tile once all are done.
    if (__syncthreads_and(done)) break;
  }
  const bool finished = __syncthreads_and(done);
  if (finished && !a.last && tid == 0) atomicOr(a.tile_done + (tile >> 5), 1u << (tile & 31u));
  if (COUNT) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      frags += __shfl_xor_sync(0xffffffffu, frags, o);
      needed += __shfl_xor_sync(0xffffffffu, needed, o);
    }
    if (lane == 0 && frags) atomicAdd(a.fragments, (unsigned long long)frags);
    if (lane == 0 && needed) atomicAdd(a.fragments + 1, (unsigned long long)needed);
  }
  if (TRAIN) {
    if (in0) {
      a.nproc[pix] = blended0;
      a.state_t[pix] = T.x;
    }
    if (in1) {
      a.nproc[pix + 1] = blended1;
      a.state_t[pix + 1] = T.y;
    }
  }
  if (!finished && !a.last) {  // a farther slab continues these pixels
    if (in0) {
      a.state_c[pix] = make_float4(cr.x, cg.x, cb.x, ca.x);
      a.state_t[pix] = T.x;
    }
    if (in1) {
      a.state_c[pix + 1] = make_float4(cr.y, cg.y, cb.y, ca.y);
      a.state_t[pix + 1] = T.y;
    }
    return;
  }
  const auto q = [](float x) { return (unsigned char)__float2uint_rn(__saturatef(x) * 255.0f); };
  if (in0) {
    const float alpha = ca.x + T.x;
    if (a.out_rgba) reinterpret_cast<float4*>(a.out_rgba)[pix] = make_float4(cr.x, cg.x, cb.x, alpha);
    if (a.out_bgra) a.out_bgra[pix] = make_uchar4(q(cb.x), q(cg.x), q(cr.x), q(alpha));
  }
  if (in1) {
    const float alpha = ca.y + T.y;
    if (a.out_rgba) reinterpret_cast<float4*>(a.out_rgba)[pix + 1] = make_float4(cr.y, cg.y, cb.y, alpha);
    if (a.out_bgra) a.out_bgra[pix + 1] = make_uchar4(q(cb.y), q(cg.y), q(cr.y), q(alpha));
  }
}

cudaError_t launch_raster(const RasterArgs& a, cudaStream_t stream) {
  const u32 tiles = a.tiles_x * a.tiles_y;
  if (tiles == 0) return cudaSuccess;
  const bool depth = a.depth != nullptr, count = a.fragments != nullptr;
  // Two pixels per thread issue fewer instructions per pixel but keep a 64-pixel warp walking until its
  // last pixel stops: they serve frames that run beside other frames (issue-bound) and the nearest
  // slab, where pixels start at full transmittance; a farther slab, whose pixels are mostly near the
  // floor already, takes one pixel per thread when the frame has the GPU to itself.
  const bool pairs = a.lean || a.first;
  if (a.nproc && pairs)
    k_raster_pairs<false, false, true><<<tiles, kPairThreads, 0, stream>>>(a);
  else if (a.nproc)
    k_raster<false, false, true><<<tiles, kRasterThreads, 0, stream>>>(a);
  else if (pairs && depth && count)
    k_raster_pairs<true, true, false><<<tiles, kPairThreads, 0, stream>>>(a);
  else if (pairs && depth)
    k_raster_pairs<true, false, false><<<tiles, kPairThreads, 0, stream>>>(a);
  else if (pairs && count)
    k_raster_pairs<false, true, false><<<tiles, kPairThreads, 0, stream>>>(a);
  else if (pairs)
    k_raster_pairs<false, false, false><<<tiles, kPairThreads, 0, stream>>>(a);
  else if (depth && count)
    k_raster<true, true, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  else if (depth)
    k_raster<true, false, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  else if (count)
    k_raster<false, true, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  else
    k_raster<false, false, false><<<tiles, kRasterThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Blend backward.  Per pixel the forward sum is RGB = sum_i a_i c_i T_i, A = sum_i a_i^2 T_i + T_end
// over the nproc entries it blended (nearest first), T_i = prod_{j<i} (1 - a_j).  Walking those
// entries in reverse from T_end, with T_i = T_{i+1} / (1 - a_i) and S the part of the loss gradient
// carried by everything behind entry i (S starts at T_end dL/dA):
//   dL/dc_i = a_i T_i dL/dRGB,   dL/da_i = T_i (c_i . dL/dRGB + 2 a_i dL/dA) - S / (1 - a_i),
//   S += (a_i c_i . dL/dRGB + a_i^2 dL/dA) T_i,
// and a_i = o exp(-q/2), q = d^T K d with K = M^T M the conic (M = rot_scale^-1, d = pixel - centre):
//   dL/do = dL/da e^{-q/2} =: P,  dL/dq = -o P / 2,  dq/dcentre = -2 K d,  dq/dK = (dx^2, dy^2, 2 dx dy).
// K and o are per splat, so a splat's centre and conic gradients follow from the moments of P over its
// pixels -- sum P, P dx, P dy, P dx^2, P dy^2, P dx dy -- which is what the pixels accumulate (the
// projection backward turns them into dL/dcentre = o K (sum P d) and dL/dK = -o/2 (sum P dx^2, sum P dy^2,
// 2 sum P dx dy)).
// Sums 9 values over the warp by recursive halving: after three halving steps each group of four lanes
// holds one of v[0..7] (index = lane bits 4, 3, 2), finished by two more shuffles; v[8] is summed
// alone.  14 shuffles instead of 45.  Lane 4k (k < 8) returns the total of v[k], lane 0 also *v8.
__device__ __forceinline__ float warp_sum9(float v[9], float* v8) {
  const u32 lane = threadIdx.x & 31u;
#pragma unroll
  for (int half = 4, off = 16; half >= 1; half >>= 1, off >>= 1) {
    const bool up = (lane & (u32)off) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = up ? v[i] : v[i + half];
      const float keep = up ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  float t = v[0];
  t += __shfl_xor_sync(0xffffffffu, t, 2);
  t += __shfl_xor_sync(0xffffffffu, t, 1);
  float e = v[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  *v8 = e;
  return t;
}

constexpr u32 kDirectLanes = 8;  // a record that at most this many lanes of a warp take skips the reduction

// Two horizontally adjacent pixels per thread and 8x8 warp blocks, as in k_raster_pairs: each warp walks
// only the records that can touch its block, a thread adds its two pixels' 9 values before the warp
// reduction (warp_sum9), so one reduction serves 64 pixels, and the per-pixel chain runs as packed FP32
// pairs; a record that few lanes take is added by those lanes directly.  A pixel that does not take a
// record gets G = 0, which leaves its T and S unchanged and adds zeros.
__global__ __launch_bounds__(kPairThreads, 8) void k_raster_backward(const RasterBackwardArgs a) {
  __shared__ float4 s_a[kPairBatch];  // (-cx, -cx, -cy, m00)
  __shared__ float4 s_b[kPairBatch];  // (m01, m10, m11, -)
  __shared__ float4 s_c[kPairBatch];  // (r, r, g, g)
  __shared__ float4 s_d[kPairBatch];  // (b, b, opacity, opacity)
  __shared__ u32 s_id[kPairBatch];
  __shared__ u32 s_bits[kPairWarps][kPairWords];
  __shared__ u32 s_nmax;
  const u32 tile = blockIdx.x;
  const u32 tx = tile % a.tiles_x, ty = tile / a.tiles_x;
  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 px = tx * kTile + (warp % kPairBX) * kPairBW + 2 * (lane % (kPairBW / 2));  // pair (px, px + 1)
  const u32 py = ty * kTile + (warp / kPairBX) * kPairBH + lane / (kPairBW / 2);
  const bool in0 = px < a.width && py < a.height, in1 = px + 1 < a.width && py < a.height;
  const size_t pix = (size_t)py * a.width + px;
  const float2 fx = make_float2(__fdiv_rn((float)(2 * px + 1), (float)a.width) - 1.0f,
                                __fdiv_rn((float)(2 * px + 3), (float)a.width) - 1.0f);
  const float fy = __fdiv_rn((float)(2 * py + 1), (float)a.height) - 1.0f;
  float2 Tcur = make_float2(in0 ? a.state_t[pix] : 1.0f, in1 ? a.state_t[pix + 1] : 1.0f);
  const float4 g0 = in0 ? a.grad_rgba[pix] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 g1 = in1 ? a.grad_rgba[pix + 1] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float2 gx = make_float2(g0.x, g1.x), gy = make_float2(g0.y, g1.y), gz = make_float2(g0.z, g1.z);
  const float2 gw = make_float2(g0.w, g1.w), gw2 = make_float2(2.0f * g0.w, 2.0f * g1.w);
  float2 S = __fmul2_rn(Tcur, gw);
  const float sx = 2.0f / (float)a.width, sy = 2.0f / (float)a.height;
  const float ox = (float)(2 * tx * kTile + 1) / (float)a.width - 1.0f;
  const float oy = (float)(2 * ty * kTile + 1) / (float)a.height - 1.0f;
  const float mx = 0.5f * sx, my = 0.5f * sy;
  const float kExp = -0.5f * 1.4426950408889634f;
  const float2 kExp2 = make_float2(kExp, kExp), kMinus1 = make_float2(-1.0f, -1.0f);
  for (int slab = (int)a.slabs - 1; slab >= 0; --slab) {  // farthest slab first: the reverse of the forward
    const u32 n0 = in0 ? a.nproc[(size_t)slab * a.nproc_stride + pix] : 0u;
    const u32 n1 = in1 ? a.nproc[(size_t)slab * a.nproc_stride + pix + 1] : 0u;
    u32 wmax = max(n0, n1);  // the most list entries any pixel of this warp blended
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if (tid == 0) s_nmax = 0;
    __syncthreads();
    if (lane == 0 && wmax) atomicMax(&s_nmax, wmax);
    __syncthreads();
    const uint2 tr = reinterpret_cast<const uint2*>(a.tile_range + (size_t)slab * a.range_stride)[tile];
    const u32 hi = min(tr.y, a.pair_capacity);
    const u32 first = hi - min(s_nmax, hi - min(tr.x, a.pair_capacity));  // farthest entry any pixel blended
    for (u32 lo = first; lo < hi; lo += kPairBatch) {  // farthest first: the reverse of the forward
      const u32 cnt = min((u32)kPairBatch, hi - lo);
#pragma unroll
      for (int r = 0; r < kPairLoads; ++r) {
        const u32 j = tid + r * kPairThreads;
        u32 m = 0;
        if (j < cnt) {
          const u32 id = a.pair_splat[lo + j];
          const float4* rec = a.record + 4 * (size_t)id;
          const float4 q0 = rec[REC_CENTER], q1 = rec[REC_ROW1], q3 = rec[REC_AXES], q2 = rec[REC_COLOR];
          s_a[j] = make_float4(-q0.x, -q0.x, -q0.y, q0.z);
          s_b[j] = make_float4(q0.w, q1.x, q1.y, 0.0f);
          s_c[j] = make_float4(q2.x, q2.x, q2.y, q2.y);
          s_d[j] = make_float4(q2.z, q2.z, q1.w, q1.w);
          s_id[j] = id;
          m = block_mask<kPairBW, kPairBH>(q0, q1, q3, ox, oy, sx, sy, mx, my);
        }
#pragma unroll
        for (int b = 0; b < kPairWarps; ++b) {
          const u32 bits = __ballot_sync(0xffffffffu, (m >> b) & 1u);
          if (lane == 0) s_bits[b][r * kPairWarps + warp] = bits;
        }
      }
      __syncthreads();
      for (int k = 0; k < kPairWords; ++k) {
        u32 word = s_bits[warp][k];
        while (word) {
          const u32 j = 32u * k + (u32)(__ffs(word) - 1);
          word &= word - 1u;
          const u32 kproc = hi - 1 - (lo + j);  // processing index in the forward (0 = nearest)
          if (kproc >= wmax) continue;           // behind every pixel of this warp (warp-uniform)
          const float4 A = s_a[j], B = s_b[j];
          const float2 dx = __fadd2_rn(fx, make_float2(A.x, A.y));
          const float dy = __fadd_rn(fy, A.z);
          const float wu = __fmul_rn(B.x, dy), wv = __fmul_rn(B.z, dy);
          const float u0 = __fadd_rn(__fmul_rn(A.w, dx.x), wu), u1 = __fadd_rn(__fmul_rn(A.w, dx.y), wu);
          const float v0 = __fadd_rn(__fmul_rn(B.y, dx.x), wv), v1 = __fadd_rn(__fmul_rn(B.y, dx.y), wv);
          const bool on0 = kproc < n0 && (fabsf(u0) <= 3.0f) & (fabsf(v0) <= 3.0f);
          const bool on1 = kproc < n1 && (fabsf(u1) <= 3.0f) & (fabsf(v1) <= 3.0f);
          const bool on = on0 || on1;
          float r[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
          if (on) {
            const float2 uu = make_float2(u0, u1), vv = make_float2(v0, v1);
            const float2 e = __fmul2_rn(__ffma2_rn(uu, uu, __fmul2_rn(vv, vv)), kExp2);
            const float2 G = make_float2(on0 ? exp2f(e.x) : 0.0f, on1 ? exp2f(e.y) : 0.0f);
            const float4 C = s_c[j], D = s_d[j];
            const float2 al = __fmul2_rn(make_float2(D.z, D.w), G);
            const float2 inv = make_float2(__fdividef(1.0f, fmaxf(1.0f - al.x, 1e-6f)),
                                           __fdividef(1.0f, fmaxf(1.0f - al.y, 1e-6f)));
            const float2 Ti = __fmul2_rn(Tcur, inv);
            const float2 cg = __ffma2_rn(make_float2(C.x, C.y), gx,
                                         __ffma2_rn(make_float2(C.z, C.w), gy, __fmul2_rn(make_float2(D.x, D.y), gz)));
            const float2 dLda = __ffma2_rn(__fmul2_rn(S, inv), kMinus1, __fmul2_rn(Ti, __ffma2_rn(al, gw2, cg)));
            S = __ffma2_rn(__fmul2_rn(al, __ffma2_rn(al, gw, cg)), Ti, S);
            Tcur = Ti;
            const float2 P = __fmul2_rn(dLda, G);  // dL/do of each pixel; dL/dq = -o P / 2
            const float2 dy2 = make_float2(dy, dy);
            const float2 pdx = __fmul2_rn(P, dx), pdy = __fmul2_rn(P, dy2);
            const float2 pxx = __fmul2_rn(pdx, dx), pyy = __fmul2_rn(pdy, dy2), pxy = __fmul2_rn(pdx, dy2);
            const float2 w = __fmul2_rn(al, Ti);
            const float2 wr = __fmul2_rn(w, gx), wg = __fmul2_rn(w, gy), wb = __fmul2_rn(w, gz);
            r[0] = P.x + P.y;
            r[1] = pdx.x + pdx.y;
            r[2] = pdy.x + pdy.y;
            r[3] = pxx.x + pxx.y;
            r[4] = pyy.x + pyy.y;
            r[5] = pxy.x + pxy.y;
            r[6] = wr.x + wr.y;
            r[7] = wg.x + wg.y;
            r[8] = wb.x + wb.y;
          }
          const u32 onmask = __ballot_sync(0xffffffffu, on);
          if (onmask) {
            float* dst = a.grad_rec + (size_t)s_id[j] * kGradRec;
            if (__popc(onmask) <= kDirectLanes) {  // few lanes: their own atomics beat a warp reduction
              if (on) {
#pragma unroll
                for (int q = 0; q < 9; ++q) atomicAdd(dst + q, r[q]);
              }
            } else {
              float r8;
              const float sum = warp_sum9(r, &r8);
              if ((lane & 3u) == 0) {
                const u32 idx = ((lane >> 4) & 1u) * 4u + ((lane >> 3) & 1u) * 2u + ((lane >> 2) & 1u);
                atomicAdd(dst + idx, sum);
              }
              if (lane == 0) atomicAdd(dst + 8, r8);
            }
          }
        }
      }
      __syncthreads();
    }
  }
}

cudaError_t launch_raster_backward(const RasterBackwardArgs& a, cudaStream_t stream) {
  const u32 tiles = a.tiles_x * a.tiles_y;
  if (tiles == 0) return cudaSuccess;
  k_raster_backward<<<tiles, kPairThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace gs
