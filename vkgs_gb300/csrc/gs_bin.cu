// gs_bin.cu -- (splat, tile) pairs in sorted order, then per-tile ranges after the tile sort.
//
// The reference rasterises one quad per sorted splat with the fixed-function pipeline
// (splat.vert:10-25, engine.cc:1474-1479).  Here every visible splat is listed in each 16x16 tile
// its 3-sigma quad can cover.  Pairs are emitted in ascending sorted position, so a stable sort on
// the tile id alone leaves every tile's list in the reference's draw order.
//
// Tile test: the tile's pixel-centre rectangle against the quad.  The rectangle's axes are covered by
// the quad's bounding box (the tile range); the quad's own axes by mapping the rectangle into the
// quad's unit frame p = rot_scale^-1 (x - c) and testing the p-range against [-3, 3].  Both tests are
// conservative (one pixel / a relative margin), so no pixel the rasteriser covers is ever dropped.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

struct TileRect {
  int tx0, tx1, ty0, ty1;  // inclusive; tx0 > tx1 when empty
};

__device__ __forceinline__ float pixel_ndc(int i, u32 size) { return (float)(2 * i + 1) / (float)size - 1.0f; }

// Inclusive pixel range whose centres may lie within [c - h, c + h] (NDC), padded by one pixel.
__device__ __forceinline__ void pixel_span(float c, float h, u32 size, int* lo, int* hi) {
  float a = ((c - h + 1.0f) * (float)size - 1.0f) * 0.5f;
  float b = ((c + h + 1.0f) * (float)size - 1.0f) * 0.5f;
  a = fminf(fmaxf(floorf(a) - 1.0f, -1.0f), (float)size);
  b = fmaxf(fminf(ceilf(b) + 1.0f, (float)size), -1.0f);
  *lo = (int)a < 0 ? 0 : (int)a;
  *hi = (int)b > (int)size - 1 ? (int)size - 1 : (int)b;
}

__device__ __forceinline__ TileRect tile_rect(float4 q0, float4 q3, u32 width, u32 height) {
  TileRect r{0, -1, 0, -1};
  if (!(q3.x >= 0.0f)) return r;  // not drawn
  int x0, x1, y0, y1;
  pixel_span(q0.x, q3.x, width, &x0, &x1);
  pixel_span(q0.y, q3.y, height, &y0, &y1);
  if (x0 > x1 || y0 > y1) return r;
  r.tx0 = x0 / (int)kTile;
  r.tx1 = x1 / (int)kTile;
  r.ty0 = y0 / (int)kTile;
  r.ty1 = y1 / (int)kTile;
  return r;
}

__device__ __forceinline__ void span_minmax(float m, float d0, float d1, float* lo, float* hi, float* mag) {
  const float a = m * d0, b = m * d1;
  *lo = fminf(a, b);
  *hi = fmaxf(a, b);
  *mag = fmaxf(fabsf(a), fabsf(b));
}

__device__ __forceinline__ bool tile_hit(float4 q0, float4 q1, int tx, int ty, u32 width, u32 height) {
  const int px0 = tx * (int)kTile, py0 = ty * (int)kTile;
  const int px1 = min(px0 + (int)kTile - 1, (int)width - 1), py1 = min(py0 + (int)kTile - 1, (int)height - 1);
  const float dx0 = pixel_ndc(px0, width) - q0.x, dx1 = pixel_ndc(px1, width) - q0.x;
  const float dy0 = pixel_ndc(py0, height) - q0.y, dy1 = pixel_ndc(py1, height) - q0.y;
  float l0, h0, g0, l1, h1, g1;
  span_minmax(q0.z, dx0, dx1, &l0, &h0, &g0);  // m00 * dx
  span_minmax(q0.w, dy0, dy1, &l1, &h1, &g1);  // m01 * dy
  const float eu = 1e-3f + 1e-5f * (g0 + g1);
  if (l0 + l1 > 3.0f + eu || h0 + h1 < -3.0f - eu) return false;
  span_minmax(q1.x, dx0, dx1, &l0, &h0, &g0);  // m10 * dx
  span_minmax(q1.y, dy0, dy1, &l1, &h1, &g1);  // m11 * dy
  const float ev = 1e-3f + 1e-5f * (g0 + g1);
  return !(l0 + l1 > 3.0f + ev || h0 + h1 < -3.0f - ev);
}

__global__ __launch_bounds__(kBinThreads) void k_bin(const BinArgs a) {
  __shared__ u32 s_scan[32];
  __shared__ u32 s_base;
  __shared__ u32 s_part;
  const u32 tid = threadIdx.x;
  const u32 v = min(*a.visible_count, a.n);
  const u32 nparts = (v + kBinTile - 1) / kBinTile;
  for (;;) {
    if (tid == 0) s_part = atomicAdd(a.ticket, 1u);
    __syncthreads();
    const u32 p = s_part;
    if (p >= nparts) break;
    const u32 r0 = p * kBinTile + tid * kBinItems;
    u32 id[kBinItems], cnt[kBinItems];
    float4 q0[kBinItems], q1[kBinItems];
    TileRect rect[kBinItems];
    u32 sum = 0;
#pragma unroll
    for (u32 k = 0; k < kBinItems; ++k) {
      cnt[k] = 0;
      rect[k] = TileRect{0, -1, 0, -1};
      id[k] = 0;
      if (r0 + k < v) {
        id[k] = a.index[r0 + k];
        const float4* rec = a.record + 4 * (size_t)id[k];
        q0[k] = rec[0];
        q1[k] = rec[1];
        rect[k] = tile_rect(q0[k], rec[3], a.width, a.height);
        for (int ty = rect[k].ty0; ty <= rect[k].ty1; ++ty)
          for (int tx = rect[k].tx0; tx <= rect[k].tx1; ++tx)
            cnt[k] += tile_hit(q0[k], q1[k], tx, ty, a.width, a.height) ? 1u : 0u;
      }
      sum += cnt[k];
    }
    u32 ptot;
    const u32 excl_t = block_exclusive_scan<kBinThreads>(sum, s_scan, &ptot);
    if (tid == 0) {
      const u32 excl = lookback(a.status, 1, p, a.epoch, ptot, a.err);
      s_base = excl;
      if (p == nparts - 1) {
        const u32 total = excl + ptot;
        *a.pair_total = total;
        *a.pair_count = min(total, a.pair_capacity);
        if (total > a.pair_capacity) atomicOr(a.err, ERR_CAPACITY);
      }
    }
    __syncthreads();
    u32 pos = s_base + excl_t;
#pragma unroll
    for (u32 k = 0; k < kBinItems; ++k) {
      if (!cnt[k]) continue;
      for (int ty = rect[k].ty0; ty <= rect[k].ty1; ++ty)
        for (int tx = rect[k].tx0; tx <= rect[k].tx1; ++tx)
          if (tile_hit(q0[k], q1[k], tx, ty, a.width, a.height)) {
            if (pos < a.pair_capacity) {
              a.pair_tile[pos] = (u32)ty * a.tiles_x + (u32)tx;
              a.pair_splat[pos] = id[k];
            }
            ++pos;
          }
    }
    __syncthreads();
  }
}

cudaError_t launch_bin(const BinArgs& a, cudaStream_t stream) {
  if (a.n == 0) return cudaSuccess;
  const u32 parts = (a.n + kBinTile - 1) / kBinTile;
  const int sms = a.num_sms > 0 ? a.num_sms : 1;
  const u32 grid = min(parts, (u32)sms * 8u);
  k_bin<<<grid, kBinThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

__global__ void k_tile_ranges(const u32* __restrict__ tile, const u32* __restrict__ pair_count, u32 capacity,
                              uint2* __restrict__ range) {
  const u32 P = min(*pair_count, capacity);
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += stride) {
    const u32 t = tile[i];
    if (i == 0 || tile[i - 1] != t) range[t].x = i;
    if (i == P - 1 || tile[i + 1] != t) range[t].y = i + 1;
  }
}

cudaError_t launch_tile_ranges(const u32* pair_tile, const u32* pair_count, u32 capacity, u32* tile_range,
                               int num_sms, cudaStream_t stream) {
  const int sms = num_sms > 0 ? num_sms : 1;
  const u32 grid = max(1u, min((capacity + 255) / 256, (u32)sms * 8u));
  k_tile_ranges<<<grid, 256, 0, stream>>>(pair_tile, pair_count, capacity, reinterpret_cast<uint2*>(tile_range));
  return cudaGetLastError();
}

}  // namespace gs
