// gs_sort.cu -- stable LSD radix sort of 32-bit keys carrying 32-bit values, count on the device.
//
// Replaces the third-party vulkan_radix_sort call of the reference
// (vrdxCmdSortKeyValueIndirect, src/vkgs/engine/engine.cc:1218-1219): ascending keys, values moved
// alongside, element count read from device memory.  Design:
//   * one histogram kernel reads the keys once and counts every 8-bit digit of every pass;
//   * one "onesweep" kernel per pass: CTAs take kRadixTile-key partitions in ticket order,
//     rank each key inside its warp with 8 ballots (stable: warp-striped loads, items in order),
//     publish per-digit partition counts through a decoupled look-back (bounded waits, epoch-tagged
//     status words so nothing is cleared between passes), then stage the partition in shared memory
//     in digit order so that the global scatter writes contiguous runs.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = kRadixItems;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // keys per partition
static_assert(RS_TILE == (int)kRadixTile, "partition size");
constexpr int RS_RADIX = 256;
constexpr int RS_MAX_PASSES = 4;

__global__ __launch_bounds__(256) void k_radix_histogram(const u32* __restrict__ keys, const u32* __restrict__ count_ptr,
                                                         u32 max_count, u32 begin_bit, u32 passes,
                                                         u32* __restrict__ hist, u32* __restrict__ err) {
  __shared__ u32 s_hist[2][RS_MAX_PASSES][RS_RADIX];  // two copies (even/odd warps) halve bank contention
  for (u32 i = threadIdx.x; i < 2 * RS_MAX_PASSES * RS_RADIX; i += blockDim.x) (&s_hist[0][0][0])[i] = 0;
  __syncthreads();
  u32 count = *count_ptr;
  if (count > max_count) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_CAPACITY);
    count = max_count;
  }
  u32(*h)[RS_RADIX] = s_hist[(threadIdx.x >> 5) & 1];
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const u32 k = keys[i];
    for (u32 p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (begin_bit + 8 * p)) & 0xffu], 1u);
  }
  __syncthreads();
  for (u32 i = threadIdx.x; i < passes * RS_RADIX; i += blockDim.x) {
    const u32 c = (&s_hist[0][0][0])[i] + (&s_hist[1][0][0])[i];
    if (c) atomicAdd(&hist[i], c);
  }
}

template <bool HAS_VALUES>
__global__ __launch_bounds__(RS_THREADS, 4) void k_radix_onesweep(
    const u32* __restrict__ keys_in, u32* __restrict__ keys_out, const u32* __restrict__ vals_in,
    u32* __restrict__ vals_out, const u32* __restrict__ count_ptr, u32 max_count, const u32* __restrict__ hist,
    u64* __restrict__ status, u32* __restrict__ ticket, u32 epoch, u32 shift, u32* __restrict__ err) {
  __shared__ uint2 s_stage[RS_TILE];   // (key, value) in digit order
  __shared__ u32 s_whist[RS_WARPS][RS_RADIX];
  __shared__ u32 s_goff[RS_RADIX];    // exclusive scan of the global digit histogram
  __shared__ u32 s_delta[RS_RADIX];   // output position minus staged position, per digit
  __shared__ u32 s_lstart[RS_RADIX];  // start of each digit inside the staged partition
  __shared__ u32 s_scan[32];
  __shared__ u32 s_part;

  const u32 tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const u32 count = min(*count_ptr, max_count);
  const u32 nparts = (count + RS_TILE - 1) / RS_TILE;
  const u32 lt = lanemask_lt();
  u32 total;
  s_goff[tid] = block_exclusive_scan<RS_THREADS>(hist[tid], s_scan, &total);

  for (;;) {
    if (tid == 0) s_part = atomicAdd(ticket, 1u);
    __syncthreads();
    const u32 p = s_part;
    if (p >= nparts) break;
    const u32 base = p * RS_TILE;
    const u32 wbase = base + warp * (32 * RS_ITEMS);

    for (u32 i = lane; i < RS_RADIX; i += 32) s_whist[warp][i] = 0;
    u32 key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
      const u32 idx = wbase + i * 32 + lane;
      key[i] = idx < count ? keys_in[idx] : 0xffffffffu;
      if (HAS_VALUES) val[i] = idx < count ? vals_in[idx] : 0u;
    }
    __syncwarp();
    // Rank every key inside its warp: lanes holding the same digit form a match group, whose lowest
    // lane reserves the group's slots with one shared-memory atomic (items in order, lanes in order:
    // the ranking is stable).
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
      const bool valid = wbase + i * 32 + lane < count;
      const u32 d = (key[i] >> shift) & 0xffu;
      const u32 peers = match_digit8(d, valid);
      const int leader = valid ? __ffs(peers) - 1 : 0;
      u32 old = 0;
      if (valid && (int)lane == leader) old = atomicAdd(&s_whist[warp][d], (u32)__popc(peers));
      old = __shfl_sync(0xffffffffu, old, leader);
      rank[i] = old + __popc(peers & lt);
    }
    __syncthreads();

    // Thread tid owns digit tid: warp-exclusive offsets, partition total, look-back.
    u32 acc = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      const u32 c = s_whist[w][tid];
      s_whist[w][tid] = acc;
      acc += c;
    }
    const u32 excl = lookback(status + tid, RS_RADIX, p, epoch, acc, err);
    u32 ptot;
    const u32 lstart = block_exclusive_scan<RS_THREADS>(acc, s_scan, &ptot);
    s_lstart[tid] = lstart;
    s_delta[tid] = s_goff[tid] + excl - lstart;  // output position = staged position + delta[digit]
    __syncthreads();

    // Stage (key, value) pairs in digit order, then write them out: consecutive threads hold
    // consecutive staged pairs, so each digit's run leaves as contiguous stores.
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
      const u32 d = (key[i] >> shift) & 0xffu;
      const u32 lpos = s_lstart[d] + s_whist[warp][d] + rank[i];
      if (wbase + i * 32 + lane < count) s_stage[lpos] = make_uint2(key[i], HAS_VALUES ? val[i] : 0u);
    }
    __syncthreads();
    const u32 nvalid = min((u32)RS_TILE, count - base);
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
      const u32 j = tid + i * RS_THREADS;
      if (j < nvalid) {
        const uint2 kv = s_stage[j];
        const u32 pos = s_delta[(kv.x >> shift) & 0xffu] + j;
        keys_out[pos] = kv.x;
        if (HAS_VALUES) vals_out[pos] = kv.y;
      }
    }
    __syncthreads();
  }
}

// The failure path of a bounded wait, for tests: partition 1 looks back at partition 0, which never
// publishes (its status word stays zero, an epoch no pass uses), so the wait gives up after kMaxSpins
// polls, records ERR_TIMEOUT and the kernel returns.
__global__ void k_wait_selftest(u64* status, u32* err) {
  if (blockIdx.x == 0 && threadIdx.x == 0) lookback(status, 1, 1, 0x5e1f7e57u, 1u, err);
}

cudaError_t launch_wait_selftest(u64* status, u32* err, cudaStream_t stream) {
  k_wait_selftest<<<1, 32, 0, stream>>>(status, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Host side.

u32 radix_passes(u32 begin_bit, u32 end_bit) { return (end_bit - begin_bit + 7) / 8; }

size_t radix_status_words(u32 max_count) {
  const size_t parts = ((size_t)max_count + RS_TILE - 1) / RS_TILE;
  return (parts ? parts : 1) * RS_RADIX;
}

cudaError_t radix_sort(const RadixSortArgs& a, cudaStream_t stream) {
  const u32 passes = radix_passes(a.begin_bit, a.end_bit);
  if (passes == 0 || passes > RS_MAX_PASSES) return cudaErrorInvalidValue;
  // control = hist[4][256] + tickets[4]
  cudaError_t e = cudaMemsetAsync(a.control, 0, kRadixControlBytes, stream);
  if (e != cudaSuccess) return e;
  u32* hist = a.control;
  u32* tickets = a.control + RS_MAX_PASSES * RS_RADIX;
  const int sms = a.num_sms > 0 ? a.num_sms : 1;
  const u32 max_parts = (a.max_count + RS_TILE - 1) / RS_TILE;
  const u32 hist_grid = (u32)min(max((a.max_count + 256 * 16 - 1) / (256 * 16), 1u), (u32)sms * 4u);
  k_radix_histogram<<<hist_grid, 256, 0, stream>>>(a.keys, a.count, a.max_count, a.begin_bit, passes, hist, a.err);
  // One CTA per partition: finished CTAs free their slot for the next partition's loads, so load,
  // rank and scatter phases of different partitions overlap on every SM.
  const u32 grid = (a.lean && kLeanSortCtasPerSm) ? max(1u, min(max_parts, (u32)sms * kLeanSortCtasPerSm))
                                                  : max(1u, max_parts);
  u32 *ks = a.keys, *vs = a.values, *kd = a.keys_alt, *vd = a.values_alt;
  for (u32 p = 0; p < passes; ++p) {
    if (a.values)
      k_radix_onesweep<true><<<grid, RS_THREADS, 0, stream>>>(ks, kd, vs, vd, a.count, a.max_count, hist + p * RS_RADIX,
                                                              a.status, tickets + p, a.epoch + p,
                                                              a.begin_bit + 8 * p, a.err);
    else
      k_radix_onesweep<false><<<grid, RS_THREADS, 0, stream>>>(ks, kd, nullptr, nullptr, a.count, a.max_count,
                                                               hist + p * RS_RADIX, a.status, tickets + p,
                                                               a.epoch + p, a.begin_bit + 8 * p, a.err);
    u32* t = ks;
    ks = kd;
    kd = t;
    t = vs;
    vs = vd;
    vd = t;
  }
  return cudaGetLastError();
}

}  // namespace gs
