// gs_bin.cu -- (splat, tile) pairs in draw order, grouped by tile.
//
// The reference draws one quad per sorted splat with the fixed-function rasteriser
// (splat.vert:10-25, engine.cc:1474-1479); the blend order of every pixel is the sorted order.  Here
// each 16x16 tile receives the list of splats whose 3-sigma quad can cover one of its pixel centres:
//   1. count : per sorted splat, the number of tiles its quad reaches -> count[r]
//   2. scan  : exclusive scan of count[] -> first[r] and the pair total P (reduce-then-scan, no waits)
//   3. emit  : each warp lists the row spans of 32 consecutive sorted splats in shared memory and its
//              lanes take consecutive pairs (span found by binary search), storing them coalesced at
//              [first[r0], ...): pairs leave in ascending sorted position, and a splat covering
//              thousands of tiles is spread over the whole warp
//   4. a stable radix sort on the tile id alone (gs_sort.cu) then groups them by tile without
//      disturbing that order, and tile ranges are read off the sorted tile ids.
// Everything runs over one depth slab of the sorted splats at a time (sorted positions [lo, hi)); from
// the second slab on, tiles that an earlier slab finished (tile_done bitmap) receive no pairs.
// The tile test is exact up to a small margin: the quad (corners c +- a +- b) is clipped to each tile
// row's band of pixel centres and the tile columns its x-extent reaches are taken; the margin only
// ever adds pairs.  count and emit evaluate the same footprint arithmetic (this unit is compiled
// without FMA contraction) and emit checks that every splat produced exactly its counted pairs.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

constexpr u32 kCountThreads = 256;
constexpr u32 kEmitThreads = 256;
constexpr u32 kEmitWarps = kEmitThreads / 32;
constexpr u32 kScanThreads = 256;
constexpr u32 kScanItems = 16;
constexpr u32 kScanTile = kScanThreads * kScanItems;  // counts per scan block
constexpr float kMarginPx = 0.25f;
constexpr u32 kGiantPairs = 128;    // splats with more pairs are expanded by a whole CTA (k_bin_giants)
constexpr u32 kGiantThreads = 256;
constexpr u32 kGiantRows = 1024;    // row prefix held in shared memory per pass

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

// Loads the splat's raster record; false when it is not drawn.
__device__ __forceinline__ bool footprint(const float4* __restrict__ record, u32 id, const TargetGeom& g,
                                          Footprint& f) {
  const float4* r = record + 4 * (size_t)id;
  const float4 q2 = __ldg(r + 2);
  if (!(q2.w > 0.0f)) return false;
  const float4 q0 = __ldg(r + 0), q3 = __ldg(r + 3);
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

// 1. pairs per sorted splat
__global__ __launch_bounds__(kCountThreads) void k_bin_count(const BinArgs a) {
  const SlabBounds sb = slab(a);
  const TargetGeom g = target_geom(a);
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 r = sb.lo + blockIdx.x * blockDim.x + threadIdx.x; r < sb.hi; r += stride) {
    Footprint f;
    u32 c = 0;
    if (footprint(a.record, __ldg(a.index + r), g, f))
      c = a.tile_done ? footprint_open_pairs(f, g, a.tile_done) : footprint_pairs(f, g);
    a.count[r] = c;
    if (c > kGiantPairs) a.giant_list[atomicAdd(a.giant_count, 1u)] = r;
  }
}

// 2a. per-block sums of count[]
__global__ __launch_bounds__(kScanThreads) void k_bin_reduce(const BinArgs a) {
  __shared__ u32 s_scan[32];
  const SlabBounds sb = slab(a);
  const u32 base = sb.lo + blockIdx.x * kScanTile;
  if (base >= sb.hi) return;
  u32 s = 0;
#pragma unroll
  for (u32 i = 0; i < kScanItems; ++i) {
    const u32 r = base + i * kScanThreads + threadIdx.x;
    s += r < sb.hi ? a.count[r] : 0u;
  }
  u32 total;
  block_exclusive_scan<kScanThreads>(s, s_scan, &total);
  if (threadIdx.x == 0) a.block_sum[blockIdx.x] = total;
}

// 2b. exclusive scan of the block sums (one CTA), the pair total and the capacity check
__global__ __launch_bounds__(1024) void k_bin_scan_blocks(const BinArgs a) {
  __shared__ u32 s_scan[32];
  __shared__ u32 s_carry;
  const SlabBounds sb = slab(a);
  const u32 nblocks = (sb.hi - sb.lo + kScanTile - 1) / kScanTile;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (u32 b0 = 0; b0 < nblocks; b0 += 1024) {
    const u32 b = b0 + threadIdx.x;
    const u32 x = b < nblocks ? a.block_sum[b] : 0u;
    u32 sum;
    const u32 excl = block_exclusive_scan<1024>(x, s_scan, &sum);
    if (b < nblocks) a.block_sum[b] = s_carry + excl;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += sum;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const u32 P = s_carry;
    *a.slab_pairs = P;
    *a.pair_count = min(P, a.pair_capacity);
    atomicMax(a.pair_total, P);
    *a.pair_sum += P;
    if (P > a.pair_capacity) atomicOr(a.err, ERR_CAPACITY);
  }
}

// 2c. count[] -> exclusive prefix (first pair of each splat), in place
__global__ __launch_bounds__(kScanThreads) void k_bin_scan(const BinArgs a) {
  __shared__ u32 s_scan[32];
  __shared__ u32 s_vals[kScanTile];
  const SlabBounds sb = slab(a);
  const u32 base = sb.lo + blockIdx.x * kScanTile;
  if (base >= sb.hi) return;
  // blocked arrangement: thread t owns elements [t*items, (t+1)*items) of the block
  for (u32 i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    const u32 r = base + i;
    s_vals[i] = r < sb.hi ? a.count[r] : 0u;
  }
  __syncthreads();
  u32 x[kScanItems], s = 0;
#pragma unroll
  for (u32 i = 0; i < kScanItems; ++i) {
    x[i] = s_vals[threadIdx.x * kScanItems + i];
    s += x[i];
  }
  u32 total;
  u32 run = a.block_sum[blockIdx.x] + block_exclusive_scan<kScanThreads>(s, s_scan, &total);
#pragma unroll
  for (u32 i = 0; i < kScanItems; ++i) {
    s_vals[threadIdx.x * kScanItems + i] = run;
    run += x[i];
  }
  __syncthreads();
  for (u32 i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    const u32 r = base + i;
    if (r < sb.hi) a.count[r] = s_vals[i];
  }
}

constexpr u32 kSpanBuf = 128;  // row spans per warp and window

// Walks the (splat, tile) pairs of 32 consecutive sorted splats (lane = splat; ok = drawn) in sorted
// order -- splat by splat, row-major inside a splat -- 32 pairs per step, and calls
// fn(has, tile, owner_lane, j) on every lane of the warp for each step (j = the pair's index among the
// 32 splats' pairs); returns the number of pairs.  The splats' row spans are listed
// in shared memory (span = one tile row of one splat) with an exclusive prefix of their widths, so a
// lane finds the span of pair j by binary search and no lane expands a footprint serially: a splat
// that covers thousands of tiles costs the whole warp as much as that many small splats.
// s_span: 2 * (kSpanBuf + 1) words of this warp's shared memory.  Whole warp.
template <class F>
__device__ __forceinline__ u32 for_each_pair(const Footprint& f, bool ok, const TargetGeom& g, u32* s_span, F&& fn) {
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
  u32 done = 0;  // pairs of earlier windows
  for (u32 rw0 = 0; rw0 < total_rows; rw0 += kSpanBuf) {
    const u32 i0 = max(rw0, rfirst), i1 = min(rfirst + nrows, rw0 + kSpanBuf);
    for (u32 i = i0; i < i1; ++i) {
      const int ty = f.ty0 + (int)(i - rfirst);
      int tx0, tx1;
      footprint_cols(f, g, ty, tx0, tx1);
      s_tile[i - rw0] = ((u32)(ty * (int)g.tiles_x + max(tx0, 0)) << 5) | lane;
      s_pfx[i - rw0] = (u32)max(0, tx1 - tx0 + 1);  // width for now
    }
    __syncwarp();
    const u32 m = min(kSpanBuf, total_rows - rw0);
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
    for (u32 j0 = 0; j0 < pairs; j0 += 32) {
      const u32 j = j0 + lane;
      const bool has = j < pairs;
      u32 tile = 0, owner = 0;
      if (has) {
        u32 lo = 0, hi = m;  // last span with s_pfx[span] <= j
        while (hi - lo > 1) {
          const u32 mid = (lo + hi) >> 1;
          if (s_pfx[mid] <= j) lo = mid;
          else hi = mid;
        }
        const u32 e = s_tile[lo];
        tile = (e >> 5) + (j - s_pfx[lo]);
        owner = e & 31u;
      }
      fn(has, tile, owner, done + j);
    }
    done += pairs;
    __syncwarp();
  }
  return done;
}

// 3. emission: warp w walks 32 consecutive sorted splats' pairs -- splat by splat, row-major inside a
//    splat -- with the span list of for_each_pair, drops pairs of finished tiles, and stores the rest
//    coalesced into the group's contiguous output range [first[r0], ...): pairs leave in ascending
//    sorted position.
__global__ __launch_bounds__(kEmitThreads) void k_bin_emit(const BinArgs a) {
  __shared__ u32 s_spans[kEmitWarps][2 * (kSpanBuf + 1)];
  const u32 warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const SlabBounds sb = slab(a);
  const u32 P = *a.slab_pairs;
  const TargetGeom g = target_geom(a);
  const u32 gwarps = gridDim.x * kEmitWarps;
  const u32 lt = lanemask_lt();
  for (u32 r0 = sb.lo + (blockIdx.x * kEmitWarps + warp) * 32; r0 < sb.hi; r0 += gwarps * 32) {
    const u32 gfirst = a.count[r0];  // exclusive prefix after the scan
    const u32 rl = min(r0 + 32u, sb.hi);
    const u32 gend = rl < sb.hi ? a.count[rl] : P;
    if (gfirst == gend) continue;  // no open pair in this group (warp-uniform)
    const u32 r = r0 + lane;
    Footprint f;
    bool ok = false;
    u32 id = 0, giant = 0;
    if (r < sb.hi) {
      const u32 mine = (r + 1 < sb.hi ? a.count[r + 1] : P) - a.count[r];
      if (mine > kGiantPairs) {
        giant = mine;  // k_bin_giants writes these
      } else {
        id = __ldg(a.index + r);
        ok = footprint(a.record, id, g, f);
      }
    }
    // giant pairs of the lanes before this one: the gaps their ranges leave in the group's output
    u32 gincl = giant;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 y = __shfl_up_sync(0xffffffffu, gincl, o);
      if (lane >= (u32)o) gincl += y;
    }
    const u32 gexcl = gincl - giant, gtotal = __shfl_sync(0xffffffffu, gincl, 31);
    u32 kept = 0;  // pairs of non-giant splats written so far
    for_each_pair(f, ok, g, s_spans[warp], [&](bool has, u32 tile, u32 owner, u32) {
      const u32 oid = __shfl_sync(0xffffffffu, id, owner);
      const u32 gap = __shfl_sync(0xffffffffu, gexcl, owner);
      const bool keep = has && !(a.tile_done && tile_is_done(a.tile_done, tile));
      const u32 ballot = __ballot_sync(0xffffffffu, keep);
      const u32 pos = gfirst + gap + kept + __popc(ballot & lt);
      if (keep && pos < a.pair_capacity) {
        a.pair_tile[pos] = tile;
        a.pair_splat[pos] = oid;
      }
      kept += __popc(ballot);
    });
    if (lane == 0 && gfirst + gtotal + kept != gend) atomicOr(a.err, ERR_INTERNAL);  // count and emit disagree
  }
}

// 3b. giants: one CTA per splat with more than kGiantPairs pairs.  Its rows' spans are listed in
//     shared memory with a block-wide prefix, every thread takes pairs j = tid, tid + 256, ... and
//     finds its row by binary search, and open pairs are packed into the splat's output range (the
//     order inside one splat's range is free: a splat meets each tile once, and the stable tile sort
//     only orders pairs of different splats).
__global__ __launch_bounds__(kGiantThreads) void k_bin_giants(const BinArgs a) {
  __shared__ u32 s_pfx[kGiantRows + 1];
  __shared__ u32 s_base[kGiantRows];
  __shared__ u32 s_scan[32];
  __shared__ u32 s_cursor;
  const SlabBounds sb = slab(a);
  const u32 P = *a.slab_pairs;
  const u32 ng = *a.giant_count;
  const TargetGeom g = target_geom(a);
  const u32 tid = threadIdx.x, lane = tid & 31u;
  for (u32 k = blockIdx.x; k < ng; k += gridDim.x) {
    const u32 r = a.giant_list[k];
    const u32 first = a.count[r];
    const u32 end = r + 1 < sb.hi ? a.count[r + 1] : P;
    Footprint f;
    const u32 id = __ldg(a.index + r);
    footprint(a.record, id, g, f);
    if (tid == 0) s_cursor = 0;
    const u32 nrows = (u32)max(0, f.ty1 - f.ty0 + 1);
    for (u32 w0 = 0; w0 < nrows; w0 += kGiantRows) {  // windows of rows (one for any real target)
      const u32 m = min(kGiantRows, nrows - w0);
      u32 carry = 0;
      for (u32 i0 = 0; i0 < m; i0 += kGiantThreads) {
        const u32 i = i0 + tid;
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
        __syncthreads();
      }
      if (tid == 0) s_pfx[m] = carry;
      __syncthreads();
      for (u32 j0 = 0; j0 < carry; j0 += kGiantThreads) {
        const u32 j = j0 + tid;
        bool keep = false;
        u32 tile = 0;
        if (j < carry) {
          u32 lo = 0, hi = m;  // last row with s_pfx[row] <= j
          while (hi - lo > 1) {
            const u32 mid = (lo + hi) >> 1;
            if (s_pfx[mid] <= j) lo = mid;
            else hi = mid;
          }
          tile = s_base[lo] + (j - s_pfx[lo]);
          keep = !(a.tile_done && tile_is_done(a.tile_done, tile));
        }
        const u32 ballot = __ballot_sync(0xffffffffu, keep);
        u32 wbase = 0;
        if (lane == 0 && ballot) wbase = atomicAdd(&s_cursor, (u32)__popc(ballot));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        const u32 pos = first + wbase + __popc(ballot & lanemask_lt());
        if (keep && pos < end && pos < a.pair_capacity) {
          a.pair_tile[pos] = tile;
          a.pair_splat[pos] = id;
        }
      }
      __syncthreads();
    }
    if (tid == 0 && s_cursor != end - first) atomicOr(a.err, ERR_INTERNAL);  // count and emit disagree
    __syncthreads();
  }
}

// 4. tile ranges from the tile-sorted pair keys
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

size_t bin_block_sums(u32 max_splats) { return (max(max_splats, 1u) + kScanTile - 1) / kScanTile; }

cudaError_t launch_bin(const BinArgs& a, cudaStream_t stream, cudaEvent_t after_count, cudaEvent_t after_scan,
                       int num_sms) {
  if (a.n == 0) {
    if (after_count) cudaEventRecord(after_count, stream);
    if (after_scan) cudaEventRecord(after_scan, stream);
    return cudaSuccess;
  }
  const u32 sms = (u32)max(num_sms, 1);
  const u32 count_grid = min((a.n + kCountThreads - 1) / kCountThreads, sms * 16u);
  k_bin_count<<<count_grid, kCountThreads, 0, stream>>>(a);
  if (after_count) cudaEventRecord(after_count, stream);
  const u32 blocks = (u32)bin_block_sums(a.n);
  k_bin_reduce<<<blocks, kScanThreads, 0, stream>>>(a);
  k_bin_scan_blocks<<<1, 1024, 0, stream>>>(a);
  k_bin_scan<<<blocks, kScanThreads, 0, stream>>>(a);
  if (after_scan) cudaEventRecord(after_scan, stream);
  const u32 emit_grid = min((a.n + kEmitThreads - 1) / kEmitThreads, sms * 8u);
  k_bin_emit<<<emit_grid, kEmitThreads, 0, stream>>>(a);
  k_bin_giants<<<sms * 2u, kGiantThreads, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_tile_ranges(const u32* pair_tile, const u32* pair_count, u32 capacity, u32* tile_range,
                               int num_sms, cudaStream_t stream) {
  const u32 grid = max(1u, min((capacity + 255) / 256, (u32)max(num_sms, 1) * 8u));
  k_tile_ranges<<<grid, 256, 0, stream>>>(pair_tile, pair_count, capacity, reinterpret_cast<uint2*>(tile_range));
  return cudaGetLastError();
}

}  // namespace gs
