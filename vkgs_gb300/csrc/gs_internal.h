// gs_internal.h -- host-side declarations shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "gs_common.cuh"

namespace gs {

// ---- radix sort (gs_sort.cu) ----
constexpr size_t kRadixControlBytes = (4 * 256 + 4) * sizeof(uint32_t);
constexpr u32 kRadixItems = 16;                      // keys per thread and partition
constexpr u32 kRadixTile = 256 * kRadixItems;        // keys per partition

struct RadixSortArgs {
  u32* keys;          // in/out (even pass count) -- see radix_sort
  u32* values;        // may be null
  u32* keys_alt;      // ping-pong buffers, max_count words
  u32* values_alt;
  const u32* count;   // device word
  u32 max_count;
  u32 begin_bit, end_bit;
  u32* control;       // kRadixControlBytes, cleared by radix_sort
  u64* status;        // radix_status_words(max_count) words, epoch-tagged
  u32 epoch;          // first epoch; passes use epoch .. epoch + passes - 1 (never 0)
  u32* err;           // device error word
  int num_sms;
  int lean;           // frames run concurrently: at most kLeanSortCtasPerSm CTAs per SM (0: one per partition)
};
constexpr u32 kLeanSortCtasPerSm = 1;

u32 radix_passes(u32 begin_bit, u32 end_bit);
size_t radix_status_words(u32 max_count);
// Sorts keys[0..*count) (and values) on bits [begin_bit, end_bit).  After an odd number of passes the
// result lies in keys_alt / values_alt.
cudaError_t radix_sort(const RadixSortArgs& a, cudaStream_t stream);
// One look-back wait that runs out (status: 2 zeroed words, err: zeroed word); for tests.
cudaError_t launch_wait_selftest(u64* status, u32* err, cudaStream_t stream);

// ---- cull + key + compaction + projection (gs_cull.cu) ----
constexpr u32 kCullThreads = 256;
constexpr u32 kCullItems = 4;
constexpr u32 kCullTile = kCullThreads * kCullItems;

struct CullArgs {
  const float* position;
  const float* cov3d;
  const float* opacity;
  const uint16_t* sh;
  u32* key;          // compacted keys, ascending id
  u32* index;        // compacted ids
  float4* record;    // N x 4 float4 raster records, indexed by id
  float* inst_by_id; // optional N x 12 reference instance records, indexed by id
  const float* sh32; // non-null: FP32 SH (N x 48) instead of sh (the differentiable path)
  u32* visible_count;
  u64* status;       // >= ceil(N / kCullTile) words
  u32* ticket;
  u32 epoch;
  u32* err;
  int num_sms;
  int staged;        // nonzero: the shared-memory-staged kernel (when the buffers allow its bulk copies)
  int lean;          // frames run concurrently: a persistent grid of kLeanCullCtasPerSm CTAs per SM
};
constexpr u32 kCullCtasPerSm = 8, kLeanCullCtasPerSm = 3;
cudaError_t launch_cull_project(const FrameConst& fc, const CullArgs& a, cudaStream_t stream);

// The cull + projection of up to kMaxCullViews views of the same splats in one launch.
constexpr u32 kMaxCullViews = 32;
struct CullView {
  u32* key;            // compacted keys / ids of the view, ascending id
  u32* index;
  float4* record;      // N x 4 float4, indexed by id
  u32* visible_count;
  u64* status;         // >= ceil(N / kCullTile) words, cleared (epoch-tagged like CullArgs.status)
};
struct CullViewsArgs {
  const float* position;
  const float* cov3d;
  const float* opacity;
  const uint16_t* sh;
  const float* sh32;  // non-null: FP32 SH instead of sh (the differentiable path)
  u32 n;
  u32 count;  // views
  u32* ticket;
  u32 epoch;
  u32* err;
  int num_sms;
  FrameConst fc[kMaxCullViews];
  CullView view[kMaxCullViews];
};
cudaError_t launch_cull_views(const CullViewsArgs& a, cudaStream_t stream);
bool is_cull_kernel(const void* f);  // the plain path's cull kernels (the only ones reading the camera)
cudaError_t cull_stream_init();     // opts the shared-memory-staged cull into its dynamic shared memory
constexpr u32 kCullStatusSplats = 256;  // splats per look-back status word of the plain cull (its finest partition)

// Gathers instance records into sorted order and writes the indirect draw arguments.
cudaError_t launch_instances(const u32* index, const u32* visible_count, const float* inst_by_id, u32 n,
                             float* instances, u32* draw_indirect, cudaStream_t stream);

// ---- tile binning (gs_bin.cu) ----
constexpr u32 kTile = 16;            // tile edge in pixels
constexpr u32 kMaxTiles = 1u << 24;  // tile ids must stay below 2^24 (radix passes on the tile id)

// Sorted positions [lo, hi) of one depth slab: ends e_prev < e_cur are cumulative shares of V in
// 1/1024 units counted from the nearest splat (the end of the ascending sort).
struct SlabBounds {
  u32 lo, hi;
};
__host__ __device__ inline SlabBounds slab_bounds(u32 v, u32 e_prev, u32 e_cur) {
  const auto off = [v](u32 e) { return (u32)(((unsigned long long)v * e + 1023ull) >> 10); };
  return SlabBounds{v - off(e_cur), v - off(e_prev)};
}

struct BinArgs {
  const u32* index;          // sorted splat ids
  const u32* visible_count;
  const float4* record;
  u32 n;                     // launch bound for V
  u32 slab_e0, slab_e1;      // this slab's share of V (slab_bounds)
  const u32* tile_done;      // bitmap of finished tiles (they get no pairs), or null
  u32 width, height, tiles_x, tiles_y;
  u32* count;                // [n] open pairs per sorted splat (0 for giants)
  u32* diff;                 // [bin_diff_words] per-row difference counts, all zero between slabs
  u32* tile_range;           // [tiles + 1][2]: (segment start, cursor); the cursor ends at the next start
  u32* tile_order;           // [tiles] tiles by descending segment length (the per-tile sort's order)
  u32* giant_list;           // [n] sorted positions of splats with a footprint box above kGiantPairs
  u32* giant_count;          // this slab's entries in giant_list (zeroed before the frame)
  u32* pair_key;             // [capacity] sorted position per pair, grouped by tile
  u32* pair_splat;           // [capacity] splat id per pair, grouped by tile, ascending sorted position
  u32 pair_capacity;
  int stack_slabs;           // pair slots of this slab follow the earlier slabs' (all slabs' lists kept)
  u32* slab_pairs;           // out: pairs this slab needs
  u32* pair_total;           // out: max over the frame's slabs of the capacity needed (atomicMax)
  unsigned long long* pair_sum;  // out: sum over the frame's slabs
  u32* pair_peak;            // out: max over every slab since the context was last checked (atomicMax)
  u32* err;
  int lean;                  // frames run concurrently: the count and emission take fewer SM slots (below)
};

size_t bin_diff_words(u32 max_tiles_x, u32 max_tiles_y);
// count + scan, event after_scan, emit, event after_emit, per-tile sort (events may be null).
cudaError_t launch_bin(const BinArgs& a, cudaStream_t stream, cudaEvent_t after_scan, cudaEvent_t after_emit,
                       int num_sms);

// ---- raster (gs_raster.cu) ----
struct RasterArgs {
  const u32* tile_range;     // [T][2] = (begin, end) into pair_splat
  u32 pair_capacity;
  const u32* pair_splat;
  const float4* record;
  u32 width, height, tiles_x, tiles_y;
  float* out_rgba;           // may be null
  uchar4* out_bgra;          // may be null
  const float* depth;        // may be null
  float t_floor;             // blending stops once every pixel of a tile is below this transmittance
  float4* state_c;           // [H*W] running (r, g, b, a) between slabs
  float* state_t;            // [H*W] running transmittance between slabs
  u32* tile_done;            // bitmap: tiles finished by an earlier slab (set here when one finishes)
  int first, last;           // first slab: no state to load; last slab: every tile resolves
  u32* nproc;                // differentiable forward: per pixel, list entries blended (exact stop at t_floor)
  unsigned long long* fragments;  // non-null: [0] covered fragments, [1] those met while T >= t_floor
                                  // (disables the early stop)
  int lean;                  // frames run concurrently: two pixels per thread (same results)
};
cudaError_t launch_raster(const RasterArgs& a, cudaStream_t stream);

// ---- differentiable path (gs_train.cu, gs_raster.cu) ----
// per-splat blend gradient record: sums over the splat's pixels of P, P dx, P dy, P dx^2, P dy^2, P dx dy
// (P = dL/do of the pixel, d = pixel - centre) and dL/d(r, g, b); 3 words of padding
constexpr u32 kGradRec = 12;
struct RasterBackwardArgs {
  const u32* tile_range;     // slab k's at tile_range + k * range_stride
  u32 range_stride;
  u32 slabs;
  u32 pair_capacity;
  const u32* pair_splat;
  const float4* record;
  u32 width, height, tiles_x, tiles_y;
  const float* state_t;      // final transmittance per pixel
  const u32* nproc;          // list entries blended per pixel, slab k's at nproc + k * nproc_stride
  u32 nproc_stride;
  const float4* grad_rgba;   // dL/d(pixel)
  float* grad_rec;           // [N][kGradRec], accumulated
};
cudaError_t launch_raster_backward(const RasterBackwardArgs& a, cudaStream_t stream);

struct TrainArgs {
  const float* means;
  const float* log_scales;
  const float* quats;
  const float* opacity_logits;
  const float* sh;
  u32 n;
  float* position;  // activated (forward)
  float* cov3d;
  float* opacity;
  float* g_means;         // backward outputs (added into)
  float* g_log_scales;
  float* g_quats;
  float* g_opacity_logits;
  float* g_sh;
};
cudaError_t launch_activate(const TrainArgs& a, cudaStream_t stream);

// The views of one differentiable step: camera constants and blend gradient records (kGradRec per splat).
constexpr u32 kMaxTrainViews = 32;
struct TrainViews {
  u32 count;
  FrameConst fc[kMaxTrainViews];
  const float* grad_rec[kMaxTrainViews];
  float vm[kMaxTrainViews][16];  // view * model, row-major (row r, column c at [4 r + c])
};
// Adds the raw-parameter gradients of all views into a.g_* (one kernel: no atomics).
cudaError_t launch_project_backward(const TrainViews& views, const TrainArgs& a, cudaStream_t stream);

// ---- loader (gs_ply.cu) ----
struct PlyOffsets {
  u32 v[60];
};
cudaError_t launch_parse_ply(const float* rows, u32 count, const PlyOffsets& off, float* position, float* cov3d,
                             float* opacity, uint16_t* sh, cudaStream_t stream);

// ---- camera constants (gs_api.cu) ----
void frame_constants(const float projection[16], const float view[16], const float model[16], const float eye[3],
                     u32 width, u32 height, u32 n, FrameConst* out);

}  // namespace gs
