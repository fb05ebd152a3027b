// gs_bin.cu -- per-tile lists of (splat, tile) pairs in draw order.
//
// The reference draws one quad per sorted splat with the fixed-function rasteriser
// (splat.vert:10-25, engine.cc:1474-1479); the blend order of every pixel is the sorted order.  Here
// each 16x16 tile receives the list of splats whose 3-sigma quad can cover one of its pixel centres,
// ascending in sorted position.  Everything runs over one depth slab of the sorted splats at a time
// (sorted positions [lo, hi)); from the second slab on, tiles that an earlier slab finished
// (tile_done bitmap) receive no pairs.  Per slab:
//   1. count : per splat, its row spans (one tile row of the quad's footprint) enter a per-row
//              difference array of tile counts (shared memory, then global atomics); splats whose
//              footprint box spans more than kGiantPairs tiles are listed as giants and counted by
//              one CTA each (k_bin_giant_count)
//   2. scan  : one CTA turns the difference rows into tile counts and an exclusive scan over tiles:
//              tile t owns pair slots [start_t, start_{t+1}), its cursor starts at start_t (with
//              stacked slabs -- the differentiable forward keeps every slab's lists for its
//              backward -- the slots start after the earlier slabs' pairs)
//   3. emit  : warps expand 32 sorted splats' pairs (span lists, giants by whole CTAs) and append the
//              splat's sorted position to its tile's segment through the cursor (atomicAdd): each
//              segment holds the right set of splats in arbitrary order
//   4. sort  : one CTA per tile, longest segments first, sorts its segment by sorted position
//              (comparison ranks for short segments, a one-pass bucket sort over the segment's key
//              range otherwise: the keys are distinct) and writes the splat ids; a tile whose cursor
//              did not end exactly at its segment end fails the self-check.
// The tile test is exact up to a small margin: the quad (corners c +- a +- b) is clipped to each tile
// row's band of pixel centres and the tile columns its x-extent reaches are taken; the margin only
// ever adds pairs.  count and emit evaluate the same footprint arithmetic (this unit is compiled
// without FMA contraction).
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

constexpr u32 kCountThreads = 512;
constexpr u32 kCountSmemWords = 12 * 1024;  // difference rows held in shared memory up to this size
constexpr u32 kEmitThreads = 256;
constexpr u32 kEmitWarps = kEmitThreads / 32;
constexpr float kMarginPx = 0.25f;
constexpr u32 kGiantPairs = 128;    // splats whose footprint box spans more tiles go to the CTA kernels
constexpr u32 kGiantThreads = 256;
constexpr u32 kGiantRows = 1024;    // row prefix held in shared memory per window
constexpr u32 kSortThreads = 256;
constexpr u32 kSortWarps = kSortThreads / 32;
constexpr u32 kSortChunk = 3072;    // segments up to this length are sorted in shared memory
constexpr u32 kSortItems = kSortChunk / kSortThreads;
constexpr u32 kSortSmall = 64;      // segments up to this length are ranked by direct comparison
constexpr u32 kSortLogBuckets = 12;

// The quad of one splat prepared for row clipping: corners in order and inverse edge slopes.
struct Footprint {
  float vx[4], vy[4], dxdy[4];
  int ty0, ty1;  // tile rows it may reach (empty when ty0 > ty1)
};

struct TargetGeom {
  u32 width, height, tiles_x;
  float inv_w, inv_h;  // 1/W, 1/H
};

__device__ __forceinline__ TargetGeom target_geom(const BinArgs& a) {
  return TargetGeom{a.width, a.height, a.tiles_x, 1.0f / (float)a.width, 1.0f / (float)a.height};
}

// Inclusive range of pixel indices whose centres (2i+1)/size - 1 lie in [lo, hi] (NDC), clamped.
__device__ __forceinline__ void pixel_range(float lo, float hi, u32 size, int& i0, int& i1) {
  const float s = (float)size;
  float a = ceilf(((lo + 1.0f) * s - 1.0f) * 0.5f);
  float b = floorf(((hi + 1.0f) * s - 1.0f) * 0.5f);
  a = fminf(fmaxf(a, 0.0f), s);
  b = fminf(fmaxf(b, -1.0f), s - 1.0f);
  i0 = (int)a;
  i1 = (int)b;
}

// Loads the splat's centre and axes (the record's first 32 bytes); false when it is not drawn.
__device__ __forceinline__ bool footprint(const float4* __restrict__ record, u32 id, const TargetGeom& g,
                                          Footprint& f) {
  const float4* r = record + 4 * (size_t)id;
  const float4 q0 = __ldg(r + REC_CENTER);
  if (!(q0.x <= 3.0e38f)) return false;  // +inf: not drawn
  const float4 q3 = __ldg(r + REC_AXES);
  const float cx = q0.x, cy = q0.y;
  const float ax = 3.0f * q3.x, ay = 3.0f * q3.y, bx = 3.0f * q3.z, by = 3.0f * q3.w;
  f.vx[0] = cx - ax - bx, f.vy[0] = cy - ay - by;
  f.vx[1] = cx + ax - bx, f.vy[1] = cy + ay - by;
  f.vx[2] = cx + ax + bx, f.vy[2] = cy + ay + by;
  f.vx[3] = cx - ax + bx, f.vy[3] = cy - ay + by;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int n = (k + 1) & 3;
    f.dxdy[k] = (f.vx[n] - f.vx[k]) / (f.vy[n] - f.vy[k]);  // +-inf/NaN for horizontal edges: never used
  }
  const float h = fabsf(ay) + fabsf(by) + 2.0f * kMarginPx * g.inv_h;
  int y0, y1;
  pixel_range(cy - h, cy + h, g.height, y0, y1);
  f.ty0 = y0 / (int)kTile;
  f.ty1 = y1 < y0 ? f.ty0 - 1 : y1 / (int)kTile;
  return true;
}

__device__ __forceinline__ void clip_edge(const Footprint& f, int k, float y, float& xmin, float& xmax) {
  const int n = (k + 1) & 3;
  if ((f.vy[k] - y) * (f.vy[n] - y) < 0.0f) {
    const float x = f.vx[k] + (y - f.vy[k]) * f.dxdy[k];
    xmin = fminf(xmin, x);
    xmax = fmaxf(xmax, x);
  }
}

// Tile columns [tx0, tx1] of tile row ty reached by the quad (empty when tx0 > tx1).
__device__ __forceinline__ void footprint_cols(const Footprint& f, const TargetGeom& g, int ty, int& tx0, int& tx1) {
  const int r0 = ty * (int)kTile, r1 = min(r0 + (int)kTile - 1, (int)g.height - 1);
  const float m = 2.0f * kMarginPx * g.inv_h;
  const float ya = (float)(2 * r0 + 1) * g.inv_h - 1.0f - m;
  const float yb = (float)(2 * r1 + 1) * g.inv_h - 1.0f + m;
  float xmin = 3.0e38f, xmax = -3.0e38f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (f.vy[k] >= ya && f.vy[k] <= yb) {
      xmin = fminf(xmin, f.vx[k]);
      xmax = fmaxf(xmax, f.vx[k]);
    }
    clip_edge(f, k, ya, xmin, xmax);
    clip_edge(f, k, yb, xmin, xmax);
  }
  tx0 = 0;
  tx1 = -1;
  if (!(xmin <= xmax)) return;
  const float mx = 2.0f * kMarginPx * g.inv_w;
  int x0, x1;
  pixel_range(xmin - mx, xmax + mx, g.width, x0, x1);
  if (x0 > x1) return;
  tx0 = x0 / (int)kTile;
  tx1 = x1 / (int)kTile;
}

__device__ __forceinline__ u32 footprint_pairs(const Footprint& f, const TargetGeom& g) {
  u32 n = 0;
  for (int ty = f.ty0; ty <= f.ty1; ++ty) {
    int tx0, tx1;
    footprint_cols(f, g, ty, tx0, tx1);
    n += (u32)max(0, tx1 - tx0 + 1);
  }
  return n;
}

// Set bits of the done bitmap over tile ids [t0, t1].
__device__ __forceinline__ u32 done_in_range(const u32* __restrict__ done, u32 t0, u32 t1) {
  u32 n = 0;
  for (u32 w = t0 >> 5; w <= (t1 >> 5); ++w) {
    u32 bits = __ldg(done + w);
    if (w == (t0 >> 5)) bits &= 0xffffffffu << (t0 & 31u);
    if (w == (t1 >> 5)) bits &= 0xffffffffu >> (31u - (t1 & 31u));
    n += __popc(bits);
  }
  return n;
}

__device__ __forceinline__ bool tile_is_done(const u32* __restrict__ done, u32 t) {
  return (__ldg(done + (t >> 5)) >> (t & 31u)) & 1u;
}

// pairs of the footprint whose tile is not finished
__device__ __forceinline__ u32 footprint_open_pairs(const Footprint& f, const TargetGeom& g, const u32* done) {
  u32 n = 0;
  for (int ty = f.ty0; ty <= f.ty1; ++ty) {
    int tx0, tx1;
    footprint_cols(f, g, ty, tx0, tx1);
    if (tx1 < tx0) continue;
    const u32 base = (u32)ty * g.tiles_x;
    n += (u32)(tx1 - tx0 + 1) - done_in_range(done, base + (u32)tx0, base + (u32)tx1);
  }
  return n;
}

__device__ __forceinline__ SlabBounds slab(const BinArgs& a) {
  return slab_bounds(min(*a.visible_count, a.n), a.slab_e0, a.slab_e1);
}

// Upper bound on the pairs of a footprint: its tile rows times the tile columns of its x-extent.
__device__ __forceinline__ u32 footprint_box_pairs(const Footprint& f, const TargetGeom& g) {
  if (f.ty1 < f.ty0) return 0;
  const float xmin = fminf(fminf(f.vx[0], f.vx[1]), fminf(f.vx[2], f.vx[3]));
  const float xmax = fmaxf(fmaxf(f.vx[0], f.vx[1]), fmaxf(f.vx[2], f.vx[3]));
  const float mx = 2.0f * kMarginPx * g.inv_w;
  int x0, x1;
  pixel_range(xmin - mx, xmax + mx, g.width, x0, x1);
  if (x1 < x0) return 0;
  return (u32)(f.ty1 - f.ty0 + 1) * (u32)(x1 / (int)kTile - x0 / (int)kTile + 1);
}

// Adds the open tiles of row span [tx0, tx1] of tile row ty to the difference row (diff: the row's
// tiles_x + 1 words); returns the number of open tiles.
__device__ __forceinline__ u32 add_span(u32* diff, const u32* __restrict__ done, const TargetGeom& g, u32 ty,
                                        u32 tx0, u32 tx1) {
  const u32 base = ty * g.tiles_x;
  const u32 nd = done ? done_in_range(done, base + tx0, base + tx1) : 0u;
  const u32 width = tx1 - tx0 + 1;
  if (nd == 0) {
    atomicAdd(diff + tx0, 1u);
    atomicAdd(diff + tx1 + 1, 0xffffffffu);
  } else if (nd < width) {  // the span straddles finished tiles: add its open tiles one by one
    for (u32 tx = tx0; tx <= tx1; ++tx) {
      if (tile_is_done(done, base + tx)) continue;
      atomicAdd(diff + tx, 1u);
      atomicAdd(diff + tx + 1, 0xffffffffu);
    }
  }
  return width - nd;
}

// 1. per-tile pair counts (difference rows) and per-splat open pair counts; giants listed
template <bool SMEM>
__global__ __launch_bounds__(kCountThreads) void k_bin_count(const BinArgs a) {
  extern __shared__ u32 s_diff[];
  const u32 rw = a.tiles_x + 1, dw = a.tiles_y * rw;
  u32* diff = SMEM ? s_diff : a.diff;
  if (SMEM) {
    for (u32 i = threadIdx.x; i < dw; i += blockDim.x) s_diff[i] = 0;
    __syncthreads();
  }
  const SlabBounds sb = slab(a);
  const TargetGeom g = target_geom(a);
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 r = sb.lo + blockIdx.x * blockDim.x + threadIdx.x; r < sb.hi; r += stride) {
    Footprint f;
    u32 c = 0;
    if (footprint(a.record, __ldg(a.index + r), g, f)) {
      if (footprint_box_pairs(f, g) > kGiantPairs) {
        a.giant_list[atomicAdd(a.giant_count, 1u)] = r;
      } else {
        for (int ty = f.ty0; ty <= f.ty1; ++ty) {
          int tx0, tx1;
          footprint_cols(f, g, ty, tx0, tx1);
          if (tx1 >= tx0) c += add_span(diff + (u32)ty * rw, a.tile_done, g, (u32)ty, (u32)tx0, (u32)tx1);
        }
      }
    }
    a.count[r] = c;  // 0 for giants: k_bin_giant_emit writes theirs
  }
  if (SMEM) {
    __syncthreads();
    for (u32 i = threadIdx.x; i < dw; i += blockDim.x) {
      const u32 v = s_diff[i];
      if (v) atomicAdd(a.diff + i, v);
    }
  }
}

// Row spans of one giant's footprint rows [w0, w0 + m): s_base[i] = first tile id of row i, s_pfx =
// exclusive prefix of the widths, s_pfx[m] = total.  Whole CTA.
__device__ __forceinline__ u32 giant_rows(const Footprint& f, const TargetGeom& g, u32 w0, u32 m, u32* s_pfx,
                                          u32* s_base, u32* s_scan) {
  u32 carry = 0;
  for (u32 i0 = 0; i0 < m; i0 += kGiantThreads) {
    const u32 i = i0 + threadIdx.x;
    u32 width = 0;
    if (i < m) {
      const int ty = f.ty0 + (int)(w0 + i);
      int tx0, tx1;
      footprint_cols(f, g, ty, tx0, tx1);
      width = (u32)max(0, tx1 - tx0 + 1);
      s_base[i] = (u32)ty * g.tiles_x + (u32)max(tx0, 0);
    }
    u32 tot;
    const u32 ex = block_exclusive_scan<kGiantThreads>(width, s_scan, &tot);
    if (i < m) s_pfx[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) s_pfx[m] = carry;
  __syncthreads();
  return carry;
}

// 1b. giants' tile counts: one CTA per giant, one thread per tile row
__global__ __launch_bounds__(kGiantThreads) void k_bin_giant_count(const BinArgs a) {
  const u32 ng = *a.giant_count;
  const TargetGeom g = target_geom(a);
  const u32 rw = a.tiles_x + 1;
  for (u32 k = blockIdx.x; k < ng; k += gridDim.x) {
    Footprint f;
    footprint(a.record, __ldg(a.index + a.giant_list[k]), g, f);
    for (int ty = f.ty0 + (int)threadIdx.x; ty <= f.ty1; ty += kGiantThreads) {
      int tx0, tx1;
      footprint_cols(f, g, ty, tx0, tx1);
      if (tx1 >= tx0) add_span(a.diff + (u32)ty * rw, a.tile_done, g, (u32)ty, (u32)tx0, (u32)tx1);
    }
  }
}

// Warp-aggregated slot in bucket b (< 64) of s_len: lanes with equal buckets (6 ballots) share one
// shared-memory atomic; returns the lane's slot.  Whole warp.
__device__ __forceinline__ u32 bucket_slot(u32* s_len, u32 b, bool valid) {
  const u32 lane = threadIdx.x & 31u;
  u32 peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const bool bit = (b >> k) & 1u;
    const u32 bb = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? bb : ~bb;
  }
  const int leader = valid ? __ffs(peers) - 1 : 0;
  u32 old = 0;
  if (valid && (int)lane == leader) old = atomicAdd(&s_len[b], (u32)__popc(peers));
  old = __shfl_sync(0xffffffffu, old, leader);
  return old + __popc(peers & lanemask_lt());
}

// 2. tile counts -> segments.  One CTA: warps turn difference rows into counts (and clear them; the
//    counts stay in shared memory when they fit), then an exclusive scan over the tiles in row-major
//    order sets each tile's start and cursor, and the tiles are listed longest segment first.
constexpr u32 kScanSmemTiles = 10240;
__global__ __launch_bounds__(1024) void k_bin_scan(const BinArgs a) {
  __shared__ u32 s_scan[32];
  __shared__ u32 s_len[33];
  __shared__ u32 s_cnt[kScanSmemTiles];
  const u32 tiles_x = a.tiles_x, rw = tiles_x + 1, T = tiles_x * a.tiles_y;
  // stacked slabs: this slab's pairs follow the earlier slabs' (read before thread 0 adds this slab's)
  const u32 base = a.stack_slabs ? (u32)min(*a.pair_sum, (unsigned long long)0xffffffffu) : 0u;
  u32* cnt = T <= kScanSmemTiles ? s_cnt : a.tile_order;  // tile_order is rewritten last
  const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (threadIdx.x < 33) s_len[threadIdx.x] = 0;
  for (u32 row = warp; row < a.tiles_y; row += 32) {
    u32 carry = 0;
    for (u32 c0 = 0; c0 < rw; c0 += 32) {
      const u32 c = c0 + lane;
      u32 v = 0;
      if (c < rw) {
        v = a.diff[row * rw + c];
        a.diff[row * rw + c] = 0;
      }
      u32 incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (u32)o) incl += y;
      }
      if (c < tiles_x) cnt[row * tiles_x + c] = carry + incl;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
  const u32 per = (T + 1023) / 1024;
  const u32 b = min(threadIdx.x * per, T), e = min(b + per, T);
  u32 s = 0;
  for (u32 t = b; t < e; ++t) s += cnt[t];
  u32 total;
  u32 run = base + block_exclusive_scan<1024>(s, s_scan, &total);
  for (u32 i = 0; i < per; ++i) {  // warp-uniform trip count
    const u32 t = b + i;
    const bool valid = t < e;
    const u32 c = valid ? cnt[t] : 0u;
    if (valid) {
      a.tile_range[2 * t] = run;
      a.tile_range[2 * t + 1] = run;
      run += c;
    }
    bucket_slot(s_len, 32 - __clz(c), valid);
  }
  if (threadIdx.x == 0) {
    a.tile_range[2 * T] = base + total;  // sentinel: end of the last segment
    a.tile_range[2 * T + 1] = base + total;
  }
  __syncthreads();
  // processing order of the per-tile sort: longest segments first (buckets by bit length)
  if (threadIdx.x == 0) {
    u32 acc = 0;
    for (int k = 32; k >= 0; --k) {
      const u32 c = s_len[k];
      s_len[k] = acc;
      acc += c;
    }
  }
  __syncthreads();
  for (u32 i = 0; i < per; ++i) {
    const u32 t = b + i;
    const bool valid = t < e;
    const u32 c = valid ? a.tile_range[2 * t + 2] - a.tile_range[2 * t] : 0u;
    const u32 slot = bucket_slot(s_len, 32 - __clz(c), valid);
    if (valid) a.tile_order[slot] = t;
  }
  if (threadIdx.x == 0) {
    const u32 need = (u32)min((unsigned long long)base + total, (unsigned long long)0xffffffffu);
    *a.slab_pairs = total;
    atomicMax(a.pair_total, need);
    atomicMax(a.pair_peak, need);
    *a.pair_sum += total;
    if (need > a.pair_capacity) atomicOr(a.err, ERR_CAPACITY);
  }
}

constexpr u32 kSpanBuf = 128;  // row spans per warp and window
constexpr u32 kPairBatch = 4;  // pairs per lane and step of the emission

// Walks the (splat, tile) pairs of 32 consecutive sorted splats (lane = splat; ok = drawn) in sorted
// order -- splat by splat, row-major inside a splat -- 32 * kPairBatch pairs per step, and calls
// fn(has[], tile[], owner_lane[]) on every lane of the warp for each step (lane l holds pairs
// j0 + 32 q + l, q < kPairBatch, so that the caller can keep kPairBatch memory operations in flight);
// returns the number of pairs.  The splats' row spans are listed
// in shared memory (span = one tile row of one splat) with an exclusive prefix of their widths, so a
// lane finds the span of pair j by binary search and no lane expands a footprint serially: a splat
// that covers thousands of tiles costs the whole warp as much as that many small splats.  The rows are
// clipped spread over the lanes too: each lane lists its splat's rows (owner lane, tile row), and the
// lanes clip the listed rows in turn from the quads kept in shared memory, so a warp takes about
// (its rows / 32) clip steps instead of the row count of its largest splat.
// s_span: 2 * (kSpanBuf + 1) words, s_quad: 12 x 32 floats of this warp's shared memory.  Whole warp.
template <class F>
__device__ __forceinline__ u32 for_each_pair(const Footprint& f, bool ok, const TargetGeom& g, u32* s_span,
                                             float (*s_quad)[32], F&& fn) {
  u32* s_tile = s_span;                // tile id of the span's first column << 5 | owner lane
  u32* s_pfx = s_span + kSpanBuf + 1;  // exclusive prefix of the span widths, [m] = total
  const u32 lane = threadIdx.x & 31u;
  const u32 nrows = ok ? (u32)max(0, f.ty1 - f.ty0 + 1) : 0u;
  u32 incl = nrows;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (u32)o) incl += y;
  }
  const u32 rfirst = incl - nrows;
  const u32 total_rows = __shfl_sync(0xffffffffu, incl, 31);
  if (nrows) {  // the quad, for the lanes that clip this splat's rows
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s_quad[k][lane] = f.vx[k];
      s_quad[4 + k][lane] = f.vy[k];
      s_quad[8 + k][lane] = f.dxdy[k];
    }
  }
  u32 done = 0;  // pairs of earlier windows
  for (u32 rw0 = 0; rw0 < total_rows; rw0 += kSpanBuf) {
    __syncwarp();
    // list this window's rows (owner lane, tile row), then clip them spread over the lanes
    const u32 i0 = max(rw0, rfirst), i1 = min(rfirst + nrows, rw0 + kSpanBuf);
    for (u32 i = i0; i < i1; ++i) s_tile[i - rw0] = ((u32)(f.ty0 + (int)(i - rfirst)) << 5) | lane;
    __syncwarp();
    const u32 m = min(kSpanBuf, total_rows - rw0);
    for (u32 e = lane; e < m; e += 32) {
      const u32 v = s_tile[e], owner = v & 31u;
      const int ty = (int)(v >> 5);
      Footprint fo;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        fo.vx[k] = s_quad[k][owner];
        fo.vy[k] = s_quad[4 + k][owner];
        fo.dxdy[k] = s_quad[8 + k][owner];
      }
      int tx0, tx1;
      footprint_cols(fo, g, ty, tx0, tx1);
      s_tile[e] = ((u32)(ty * (int)g.tiles_x + max(tx0, 0)) << 5) | owner;
      s_pfx[e] = (u32)max(0, tx1 - tx0 + 1);  // width for now
    }
    __syncwarp();
    // exclusive scan of the m widths in place: each lane owns kSpanBuf/32 consecutive entries
    constexpr u32 kPer = kSpanBuf / 32;
    u32 w[kPer], s = 0;
#pragma unroll
    for (u32 q = 0; q < kPer; ++q) {
      const u32 e = lane * kPer + q;
      w[q] = e < m ? s_pfx[e] : 0u;
      s += w[q];
    }
    u32 sincl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, sincl, o);
      if (lane >= (u32)o) sincl += y;
    }
    const u32 pairs = __shfl_sync(0xffffffffu, sincl, 31);
    u32 run = sincl - s;
    __syncwarp();
#pragma unroll
    for (u32 q = 0; q < kPer; ++q) {
      const u32 e = lane * kPer + q;
      if (e < m) s_pfx[e] = run;
      run += w[q];
    }
    if (lane == 0) s_pfx[m] = pairs;
    __syncwarp();
    for (u32 j0 = 0; j0 < pairs; j0 += 32 * kPairBatch) {
      bool has[kPairBatch];
      u32 tile[kPairBatch], owner[kPairBatch];
#pragma unroll
      for (u32 q = 0; q < kPairBatch; ++q) {
        const u32 j = j0 + 32 * q + lane;
        has[q] = j < pairs;
        tile[q] = 0;
        owner[q] = 0;
        if (has[q]) {
          u32 lo = 0, hi = m;  // last span with s_pfx[span] <= j
          while (hi - lo > 1) {
            const u32 mid = (lo + hi) >> 1;
            if (s_pfx[mid] <= j) lo = mid;
            else hi = mid;
          }
          const u32 e = s_tile[lo];
          tile[q] = (e >> 5) + (j - s_pfx[lo]);
          owner[q] = e & 31u;
        }
      }
      fn(has, tile, owner);
    }
    done += pairs;
    __syncwarp();
  }
  return done;
}

// 3. emission: warp w walks the pairs of 32 consecutive sorted splats with the span list of
//    for_each_pair and appends each open pair's sorted position to its tile's segment.
__global__ __launch_bounds__(kEmitThreads) void k_bin_emit(const BinArgs a) {
  __shared__ u32 s_spans[kEmitWarps][2 * (kSpanBuf + 1)];
  __shared__ float s_quads[kEmitWarps][12][32];
  const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const SlabBounds sb = slab(a);
  const TargetGeom g = target_geom(a);
  const u32 gwarps = gridDim.x * kEmitWarps;
  for (u32 r0 = sb.lo + (blockIdx.x * kEmitWarps + warp) * 32; r0 < sb.hi; r0 += gwarps * 32) {
    const u32 r = r0 + lane;
    const u32 c = r < sb.hi ? a.count[r] : 0u;
    if (__ballot_sync(0xffffffffu, c > 0) == 0) continue;  // nothing open in this group
    Footprint f;
    bool ok = false;
    if (c > 0) ok = footprint(a.record, __ldg(a.index + r), g, f);
    for_each_pair(f, ok, g, s_spans[warp], s_quads[warp], [&](const bool* has, const u32* tile, const u32* owner) {
      u32 pos[kPairBatch];
#pragma unroll
      for (u32 q = 0; q < kPairBatch; ++q) {  // all slots reserved first: the atomics overlap
        pos[q] = 0xffffffffu;
        if (has[q] && !(a.tile_done && tile_is_done(a.tile_done, tile[q])))
          pos[q] = atomicAdd(a.tile_range + 2 * tile[q] + 1, 1u);
      }
#pragma unroll
      for (u32 q = 0; q < kPairBatch; ++q)
        if (pos[q] < a.pair_capacity) a.pair_key[pos[q]] = r0 + owner[q];
    });
  }
}

// 3b. giants: one CTA per listed splat; every thread takes pairs j = tid, tid + 256, ... of the row
//     span list and finds its row by binary search.
__global__ __launch_bounds__(kGiantThreads) void k_bin_giant_emit(const BinArgs a) {
  __shared__ u32 s_pfx[kGiantRows + 1];
  __shared__ u32 s_base[kGiantRows];
  __shared__ u32 s_scan[32];
  const u32 ng = *a.giant_count;
  const TargetGeom g = target_geom(a);
  for (u32 k = blockIdx.x; k < ng; k += gridDim.x) {
    const u32 r = a.giant_list[k];
    Footprint f;
    footprint(a.record, __ldg(a.index + r), g, f);
    const u32 nrows = (u32)max(0, f.ty1 - f.ty0 + 1);
    for (u32 w0 = 0; w0 < nrows; w0 += kGiantRows) {  // windows of rows (one for any real target)
      const u32 m = min(kGiantRows, nrows - w0);
      const u32 total = giant_rows(f, g, w0, m, s_pfx, s_base, s_scan);
      for (u32 j = threadIdx.x; j < total; j += kGiantThreads) {
        u32 lo = 0, hi = m;  // last row with s_pfx[row] <= j
        while (hi - lo > 1) {
          const u32 mid = (lo + hi) >> 1;
          if (s_pfx[mid] <= j) lo = mid;
          else hi = mid;
        }
        const u32 tile = s_base[lo] + (j - s_pfx[lo]);
        if (a.tile_done && tile_is_done(a.tile_done, tile)) continue;
        const u32 pos = atomicAdd(a.tile_range + 2 * tile + 1, 1u);
        if (pos < a.pair_capacity) a.pair_key[pos] = r;
      }
      __syncthreads();
    }
  }
}

// Bucket layout of one segment's keys (distinct sorted positions): bucket(k) = (k - kmin) >> shift,
// about two buckets per key (at most 2^kSortLogBuckets), so that buckets hold very few keys.
struct Buckets {
  u32 kmin, shift, nbk;
  __device__ __forceinline__ u32 of(u32 k) const { return (k - kmin) >> shift; }
};

__device__ __forceinline__ Buckets make_buckets(u32 kmin, u32 kmax, u32 n) {
  const u32 bits = 32 - __clz(kmax - kmin);                   // bits of the key range
  const u32 lb = min(kSortLogBuckets, 33 - __clz(n - 1));     // ceil(log2 n) + 1, n >= 2
  const u32 shift = bits > lb ? bits - lb : 0;
  return Buckets{kmin, shift, ((kmax - kmin) >> shift) + 1};  // <= 2^lb buckets
}

// In place: s_cnt[0..nbk) counts -> exclusive starts, s_cnt[nbk] = total.  Whole CTA.
__device__ __forceinline__ void scan_buckets(u32* s_cnt, u32 nbk, u32* s_scan) {
  const u32 per = (nbk + kSortThreads - 1) / kSortThreads;
  const u32 b0 = min(threadIdx.x * per, nbk), b1 = min(b0 + per, nbk);
  u32 s = 0;
  for (u32 b = b0; b < b1; ++b) s += s_cnt[b];
  u32 total;
  u32 run = block_exclusive_scan<kSortThreads>(s, s_scan, &total);
  for (u32 b = b0; b < b1; ++b) {
    const u32 c = s_cnt[b];
    s_cnt[b] = run;
    run += c;
  }
  if (threadIdx.x == 0) s_cnt[nbk] = total;
  __syncthreads();
}

// Minimum and maximum over the CTA (thread values in, block values out).  Whole CTA.
__device__ __forceinline__ void block_min_max(u32& kmin, u32& kmax, u32 (*s_red)[kSortWarps]) {
  const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  kmin = __reduce_min_sync(0xffffffffu, kmin);
  kmax = __reduce_max_sync(0xffffffffu, kmax);
  if (lane == 0) {
    s_red[0][warp] = kmin;
    s_red[1][warp] = kmax;
  }
  __syncthreads();
  kmin = s_red[0][0];
  kmax = s_red[1][0];
#pragma unroll
  for (u32 w = 1; w < kSortWarps; ++w) {
    kmin = min(kmin, s_red[0][w]);
    kmax = max(kmax, s_red[1][w]);
  }
}

// 4. one CTA per tile (longest segments first): sort the segment's sorted positions ascending and
//    write the splat ids in that order.  The keys of a segment are distinct, so a one-pass bucket
//    sort needs no stability: keys are counted into about 2n buckets over the segment's key range,
//    scattered to their bucket (any order inside it), and each key's final place is its bucket's
//    start plus the keys of its bucket below it.  Up to kSortSmall keys: rank by direct comparison;
//    up to kSortChunk: everything in shared memory; longer: the same steps through the segment's
//    key and output arrays in global memory.
__global__ __launch_bounds__(kSortThreads) void k_tile_sort(const BinArgs a) {
  __shared__ u32 s_cnt[(1u << kSortLogBuckets) + 1];
  __shared__ u32 s_a[kSortChunk];
  __shared__ u32 s_b[kSortChunk];
  __shared__ u32 s_scan[32];
  __shared__ u32 s_red[2][kSortWarps];
  const u32 t = a.tile_order[blockIdx.x], tid = threadIdx.x;
  if (a.tile_done && tile_is_done(a.tile_done, t)) return;
  const u32 start = a.tile_range[2 * t], cursor = a.tile_range[2 * t + 1], end = a.tile_range[2 * t + 2];
  if (tid == 0 && cursor != end) atomicOr(a.err, ERR_INTERNAL);  // emitted pairs != counted pairs
  const u32 x = min(start, a.pair_capacity), n = min(cursor, a.pair_capacity) - x;
  if (n == 0) return;
  u32* key = a.pair_key + x;
  u32* out = a.pair_splat + x;
  if (n <= kSortSmall) {  // a key's rank by direct comparison with all the others
    const u32 k = tid < n ? key[tid] : 0u;
    if (tid < n) s_a[tid] = k;
    __syncthreads();
    if (tid < n) {
      u32 rank = 0;
      for (u32 j = 0; j < n; ++j) rank += s_a[j] < k ? 1u : 0u;
      out[rank] = __ldg(a.index + k);
    }
    return;
  }
  if (n <= kSortChunk) {
    u32 k[kSortItems], slot[kSortItems];
    u32 kmin = 0xffffffffu, kmax = 0;
#pragma unroll
    for (u32 i = 0; i < kSortItems; ++i) {
      const u32 e = tid + i * kSortThreads;
      k[i] = e < n ? key[e] : 0u;
      if (e < n) {
        kmin = min(kmin, k[i]);
        kmax = max(kmax, k[i]);
      }
    }
    block_min_max(kmin, kmax, s_red);
    const Buckets bk = make_buckets(kmin, kmax, n);
    for (u32 b = tid; b <= bk.nbk; b += kSortThreads) s_cnt[b] = 0;
    __syncthreads();
#pragma unroll
    for (u32 i = 0; i < kSortItems; ++i)
      if (tid + i * kSortThreads < n) slot[i] = atomicAdd(&s_cnt[bk.of(k[i])], 1u);
    __syncthreads();
    scan_buckets(s_cnt, bk.nbk, s_scan);
#pragma unroll
    for (u32 i = 0; i < kSortItems; ++i)
      if (tid + i * kSortThreads < n) s_a[s_cnt[bk.of(k[i])] + slot[i]] = k[i];
    __syncthreads();
#pragma unroll
    for (u32 i = 0; i < kSortItems; ++i) {
      if (tid + i * kSortThreads < n) {
        const u32 b = bk.of(k[i]), lo = s_cnt[b], hi = s_cnt[b + 1];
        u32 rank = lo;
        for (u32 j = lo; j < hi; ++j) rank += s_a[j] < k[i] ? 1u : 0u;
        s_b[rank] = k[i];
      }
    }
    __syncthreads();
    for (u32 e = tid; e < n; e += kSortThreads) out[e] = __ldg(a.index + s_b[e]);
    return;
  }
  // Longer segments: count, scatter through per-bucket cursors into the output array (after which
  // s_cnt[b] is bucket b's end and bucket b starts at s_cnt[b - 1]), place each key into the key
  // array, then gather the splat ids.
  u32 kmin = 0xffffffffu, kmax = 0;
  for (u32 e = tid; e < n; e += kSortThreads) {
    const u32 k = key[e];
    kmin = min(kmin, k);
    kmax = max(kmax, k);
  }
  block_min_max(kmin, kmax, s_red);
  const Buckets bk = make_buckets(kmin, kmax, n);
  for (u32 b = tid; b <= bk.nbk; b += kSortThreads) s_cnt[b] = 0;
  __syncthreads();
  for (u32 e = tid; e < n; e += kSortThreads) atomicAdd(&s_cnt[bk.of(key[e])], 1u);
  __syncthreads();
  scan_buckets(s_cnt, bk.nbk, s_scan);
  for (u32 e = tid; e < n; e += kSortThreads) {
    const u32 k = key[e];
    out[atomicAdd(&s_cnt[bk.of(k)], 1u)] = k;
  }
  __syncthreads();
  for (u32 e = tid; e < n; e += kSortThreads) {
    const u32 k = out[e], b = bk.of(k), lo = b ? s_cnt[b - 1] : 0u, hi = s_cnt[b];
    u32 rank = lo;
    for (u32 j = lo; j < hi; ++j) rank += out[j] < k ? 1u : 0u;
    key[rank] = k;
  }
  __syncthreads();
  for (u32 e = tid; e < n; e += kSortThreads) out[e] = __ldg(a.index + key[e]);
}

size_t bin_diff_words(u32 max_tiles_x, u32 max_tiles_y) { return (size_t)(max_tiles_x + 1) * max_tiles_y; }

cudaError_t launch_bin(const BinArgs& a, cudaStream_t stream, cudaEvent_t after_scan, cudaEvent_t after_emit,
                       int num_sms) {
  const u32 sms = (u32)max(num_sms, 1);
  const u32 tiles = a.tiles_x * a.tiles_y;
  const u32 dw = (a.tiles_x + 1) * a.tiles_y;
  // When other frames run beside this one (frames in flight, render lanes), the count and the emission
  // are launched lean -- half the count's threads, an eighth of the emission's CTAs: alone they take
  // longer (count 0.32 vs 0.24 ms on the bench workload), but they leave SM slots to the concurrent
  // frames, which gives more frames per second overall (with the lean cull and sort grids: 885 vs 869
  // frames/s with five frames in flight; 861 vs 824 with four, before the emission went 2 -> 1).
  const u32 count_threads = a.lean ? kCountThreads / 2 : kCountThreads;
  const u32 count_grid = max(1u, min((a.n + count_threads - 1) / count_threads, sms * 2u));
  if (dw <= kCountSmemWords)
    k_bin_count<true><<<count_grid, count_threads, dw * sizeof(u32), stream>>>(a);
  else
    k_bin_count<false><<<count_grid, count_threads, 0, stream>>>(a);
  k_bin_giant_count<<<sms * 2u, kGiantThreads, 0, stream>>>(a);
  k_bin_scan<<<1, 1024, 0, stream>>>(a);
  if (after_scan) cudaEventRecord(after_scan, stream);
  const u32 emit_grid = max(1u, min((a.n + kEmitThreads - 1) / kEmitThreads, sms * (a.lean ? 1u : 8u)));
  k_bin_emit<<<emit_grid, kEmitThreads, 0, stream>>>(a);
  k_bin_giant_emit<<<sms * 2u, kGiantThreads, 0, stream>>>(a);
  if (after_emit) cudaEventRecord(after_emit, stream);
  k_tile_sort<<<max(tiles, 1u), kSortThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace gs
