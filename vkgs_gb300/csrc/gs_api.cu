// gs_api.cu -- the C ABI: render context, frame orchestration, sorter, loader and camera helpers.
//
// The frame sequence replaces Engine::Impl::Draw's compute + draw recording
// (src/vkgs/engine/engine.cc:1164-1290 and DrawNormalPass 1380-1498):
//   reference                                  here
//   fill(visible_count, 0) + rank.comp          cull + key + order-preserving compaction + projection
//   vrdxCmdSortKeyValueIndirect                 onesweep radix sort of (key, index), count on device
//   fill(inverse, -1) + inverse_index.comp      (not needed: records are keyed by splat id)
//   projection.comp                             (fused into the cull pass)
//   vkCmdDrawIndexedIndirect + blend            ordered tile binning -> stable tile-id sort -> tile raster
// Nothing here synchronises the host or allocates after gs_context_create/gs_context_reserve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/vkgs_gb300.h"
#include "gs_internal.h"

using namespace gs;

namespace {

constexpr uint32_t kVersion = 1 * 10000 + 0 * 100 + 0;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// A single device allocation carved into aligned sub-buffers.
struct Carver {
  size_t offset = 0;
  char* base = nullptr;
  template <typename T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base ? base + offset : nullptr);
    offset += align_up(count * sizeof(T) + 16);
    return p;
  }
};

gs_status from_cuda(cudaError_t e) { return e == cudaSuccess ? GS_SUCCESS : GS_ERROR_CUDA; }

// Frame-local device words (cleared at the start of every frame).
enum FrameWord : u32 {
  FW_VISIBLE = 0,
  FW_PAIR_COUNT = 1,
  FW_PAIR_TOTAL = 2,
  FW_TICKET_CULL = 3,
  FW_FRAGMENTS = 4,  // u64 covered fragments at words 4..5, u64 blended fragments at 6..7
  FW_SLAB_PAIRS = 8,  // pairs of the slab being binned
  FW_PAIR_SUM = 10,   // u64 pairs over all slabs at words 10..11
  FW_GIANTS = 12,     // giant-splat list length, one word per slab (12..15)
  FW_WORDS = 16,
};

}  // namespace

struct gs_context {
  int device = 0;
  int num_sms = 1;
  u32 max_splats = 0, max_width = 0, max_height = 0, max_tiles = 0, pair_capacity = 0;
  int count_fragments = 0;
  float t_floor = 1e-4f;  // early stop: remaining contributions move no channel by more than this
  bool staged_cull = false;  // plain path: stage each cull partition in shared memory with bulk copies
  bool lean = false;         // its frames run beside other frames (viewer slots, render lanes)
  u32 epoch = 1;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  // carved buffers
  u32* frame = nullptr;  // FW_WORDS
  u32* err = nullptr;
  u32* key = nullptr;
  u32* index = nullptr;
  u32* key_alt = nullptr;
  u32* index_alt = nullptr;
  float4* record = nullptr;
  float* inst_by_id = nullptr;
  u64* cull_status = nullptr;
  u32* radix_control = nullptr;
  u64* radix_status = nullptr;
  size_t radix_status_words = 0;
  u32* bin_count = nullptr;
  u32* bin_diff = nullptr;
  u32* giant_list = nullptr;
  u32* pair_key = nullptr;
  u32* pair_splat = nullptr;
  u32* tile_range = nullptr;
  u32* tile_done = nullptr;   // bitmap over tiles, cleared per frame
  u32* tile_order = nullptr;
  // differentiable path
  float* train_pos = nullptr;      // activated splats of the last gs_train_forward
  float* train_cov = nullptr;
  float* train_opacity = nullptr;
  u32* train_nproc = nullptr;      // per slab and pixel: list entries blended
  u32 train_slabs = 1;             // depth slabs of the last differentiable forward
  const float4* train_record = nullptr;  // the records that forward drew (its backward reads them)
  // Frames recorded on this context, and which of them was the last differentiable forward: a
  // backward whose forward state (tile lists, blended counts, records) was overwritten since by another
  // frame on this context is refused instead of reading another frame's lists.
  u64 frame_gen = 0, train_gen = 0;
  // The differentiable forward uses the slab schedule from this many splats on; below it the per-slab
  // fixed cost (seven more launches, the blended-count clears) outweighs the pairs it saves (measured:
  // 200k splats at 800x800, one slab 0.86 ms per fwd+bwd step vs 0.94 ms with two; 3M splats x 16
  // views, two slabs 29.9 ms vs 32.1 ms).
  u32 train_slab_min = 1u << 20;
  float* grad_rec = nullptr;       // per splat blend gradients (kGradRec floats)
  float4* state_c = nullptr;  // running pixel sums between depth slabs
  float* state_t = nullptr;
  // batched rendering: render lanes (sub-contexts with their own scratch and stream)
  bool multi_view_cull = true;  // batched form: one k_cull_views pass for all views (else per lane)
  char* batch_arena = nullptr;  // per-view cull outputs of the batched form (see batch_buffers)
  size_t batch_bytes = 0;
  u32 batch_views = 0, batch_n = 0;
  u64 batch_gen = 0;        // writes into the batch arena (shared culls) and its reallocations
  u64 train_batch_gen = 0;  // batch_gen right after the last batched differentiable forward (0: no arena)
  u32 train_views = 0;      // views of the last batched differentiable forward
  bool batch_captured = false;  // a batched call was recorded into a stream capture with the arena
  gs_context* lane[GS_MAX_LANES] = {};
  cudaStream_t lane_stream[GS_MAX_LANES] = {};
  cudaEvent_t lane_join[GS_MAX_LANES] = {};
  cudaEvent_t batch_fork = nullptr;
  cudaEvent_t chunk_done[64] = {};  // batched render: one per shared-cull chunk (kMaxBatchViews / kCullChunk)
  u32 nlanes = 0;
  bool last_batched = false;
  u32 slab_count = 2;  // nearest 3/16 of the visible splats, then the rest
  u32 slab_end[GS_MAX_SLABS] = {192, 1024, 1024, 1024};
  size_t status_bytes_begin = 0, status_bytes_end = 0;  // epoch-tagged region (zeroed on allocation)
  // stage timing: a ring of kTimingRing frames x kFrameEvents events -- start, after cull, after the
  // depth sort, then per slab: after binning, tile sort, tile ranges and raster
  static constexpr u32 kTimingRing = 256;
  static constexpr u32 kFrameEvents = 3 + 4 * GS_MAX_SLABS;
  bool timing = false;
  cudaEvent_t* events = nullptr;
  u32 frame_slabs[kTimingRing] = {};
  u32 timed_frames = 0;  // frames recorded since enabling (may exceed the ring)

  cudaEvent_t* frame_events(u32 frame) { return events + (size_t)(frame % kTimingRing) * kFrameEvents; }
};

struct gs_sorter {
  int device = 0;
  int num_sms = 1;
  u32* err = nullptr;  // device word
};

// The context arena: every per-frame buffer at the given capacities, carved from one allocation (cv
// with a null base only measures).
static void context_layout(Carver& cv, gs_context* t, u32 max_splats, u32 max_width, u32 max_height, u32 max_pairs) {
  const u32 tiles_x = (max_width + kTile - 1) / kTile, tiles_y = (max_height + kTile - 1) / kTile;
  const u32 max_tiles = std::max(1u, tiles_x * tiles_y);
  const u32 n = std::max(1u, max_splats);
  const u32 pairs = std::max(1u, max_pairs);
  {
    t->frame = cv.take<u32>(FW_WORDS);
    t->err = cv.take<u32>(4);
    t->key = cv.take<u32>(n);
    t->index = cv.take<u32>(n);
    t->key_alt = cv.take<u32>(n);
    t->index_alt = cv.take<u32>(n);
    t->record = cv.take<float4>((size_t)n * 4);
    t->inst_by_id = cv.take<float>((size_t)n * 12);
    t->bin_count = cv.take<u32>(n);
    t->bin_diff = cv.take<u32>(bin_diff_words(tiles_x, tiles_y));
    t->giant_list = cv.take<u32>(n);
    t->tile_range = cv.take<u32>((size_t)GS_MAX_SLABS * (max_tiles + 1) * 2);  // one per slab (stacked)
    t->tile_done = cv.take<u32>((max_tiles + 31) / 32);
    t->tile_order = cv.take<u32>(max_tiles);
    t->train_pos = cv.take<float>((size_t)n * 3);
    t->train_cov = cv.take<float>((size_t)n * 6);
    t->train_opacity = cv.take<float>(n);
    t->train_nproc = cv.take<u32>((size_t)GS_MAX_SLABS * max_width * max_height);  // per slab
    t->grad_rec = cv.take<float>((size_t)n * kGradRec);
    t->state_c = cv.take<float4>((size_t)max_width * max_height);
    t->state_t = cv.take<float>((size_t)max_width * max_height);
    t->radix_control = cv.take<u32>(kRadixControlBytes / sizeof(u32));
    t->pair_key = cv.take<u32>(pairs);
    t->pair_splat = cv.take<u32>(pairs);
    t->status_bytes_begin = cv.offset;
    t->cull_status = cv.take<u64>((n + kCullStatusSplats - 1) / kCullStatusSplats);
    t->radix_status_words = radix_status_words(n);
    t->radix_status = cv.take<u64>(t->radix_status_words);
    t->status_bytes_end = cv.offset;
  }
}

static gs_status context_allocate(gs_context* c, u32 max_splats, u32 max_width, u32 max_height, u32 max_pairs) {
  const u32 tiles_x = (max_width + kTile - 1) / kTile, tiles_y = (max_height + kTile - 1) / kTile;
  const u32 max_tiles = std::max(1u, tiles_x * tiles_y);
  const u32 n = std::max(1u, max_splats);
  const u32 pairs = std::max(1u, max_pairs);
  if (max_tiles > kMaxTiles) return GS_ERROR_CAPACITY;
  Carver plan;
  gs_context probe;
  context_layout(plan, &probe, max_splats, max_width, max_height, max_pairs);
  char* arena = nullptr;
  if (cudaMalloc(&arena, plan.offset) != cudaSuccess) {
    cudaGetLastError();
    return GS_ERROR_OUT_OF_MEMORY;
  }
  if (cudaMemset(arena, 0, plan.offset) != cudaSuccess) {
    cudaFree(arena);
    return GS_ERROR_CUDA;
  }
  if (c->arena) {
    cudaDeviceSynchronize();
    cudaFree(c->arena);
  }
  Carver real;
  real.base = arena;
  context_layout(real, c, max_splats, max_width, max_height, max_pairs);
  c->arena = arena;
  c->arena_bytes = plan.offset;
  c->max_splats = n;
  c->max_width = max_width;
  c->max_height = max_height;
  c->max_tiles = max_tiles;
  c->pair_capacity = pairs;
  c->epoch = 1;
  return GS_SUCCESS;
}

namespace gs {

static void mat4_mul_host(const float a[16], const float b[16], float out[16]) {
  float r[16];
  for (int j = 0; j < 4; ++j)
    for (int i = 0; i < 4; ++i)
      r[j * 4 + i] = ((a[0 * 4 + i] * b[j * 4 + 0] + a[1 * 4 + i] * b[j * 4 + 1]) + a[2 * 4 + i] * b[j * 4 + 2]) +
                     a[3 * 4 + i] * b[j * 4 + 3];
  std::memcpy(out, r, sizeof(r));
}

// det and adjugate of a 4x4 (column-major) in double, by cofactor expansion.
static void camera_in_model_space(const float model[16], const float eye[3], float out[3]) {
  double m[4][4];  // m[row][col]
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) m[r][c] = model[c * 4 + r];
  auto minor3 = [&](int skip_r, int skip_c) {
    double s[3][3];
    for (int r = 0, rr = 0; r < 4; ++r) {
      if (r == skip_r) continue;
      for (int c = 0, cc = 0; c < 4; ++c) {
        if (c == skip_c) continue;
        s[rr][cc++] = m[r][c];
      }
      ++rr;
    }
    return s[0][0] * (s[1][1] * s[2][2] - s[1][2] * s[2][1]) - s[0][1] * (s[1][0] * s[2][2] - s[1][2] * s[2][0]) +
           s[0][2] * (s[1][0] * s[2][1] - s[1][1] * s[2][0]);
  };
  double inv[4][4];  // inv[row][col] = cofactor(col,row) / det
  double det = 0.0;
  for (int c = 0; c < 4; ++c) det += ((c & 1) ? -1.0 : 1.0) * m[0][c] * minor3(0, c);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) inv[r][c] = (((r + c) & 1) ? -1.0 : 1.0) * minor3(c, r) / det;
  const double e[4] = {eye[0], eye[1], eye[2], 1.0};
  double p[4];
  for (int r = 0; r < 4; ++r) p[r] = inv[r][0] * e[0] + inv[r][1] * e[1] + inv[r][2] * e[2] + inv[r][3] * e[3];
  for (int i = 0; i < 3; ++i) out[i] = (float)(p[i] / p[3]);
}

void frame_constants(const float projection[16], const float view[16], const float model[16], const float eye[3],
                     u32 width, u32 height, u32 n, FrameConst* fc) {
  float pv[16];
  mat4_mul_host(projection, view, pv);
  mat4_mul_host(pv, model, fc->pvm);
  std::memcpy(fc->model, model, 64);
  std::memcpy(fc->view, view, 64);
  std::memcpy(fc->proj, projection, 64);
  bool ident = true;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) ident = ident && model[c * 4 + r] == (c == r ? 1.0f : 0.0f);
  fc->model_identity = ident ? 1u : 0u;
  if (ident) {
    fc->cam_m[0] = eye[0], fc->cam_m[1] = eye[1], fc->cam_m[2] = eye[2];
  } else {
    camera_in_model_space(model, eye, fc->cam_m);
  }
  fc->lpx = 1.0f / (float)width / (float)width;
  fc->lpy = 1.0f / (float)height / (float)height;
  fc->width = width;
  fc->height = height;
  fc->n = n;
}

}  // namespace gs

extern "C" {

const char* gs_status_string(gs_status s) {
  switch (s) {
    case GS_SUCCESS: return "success";
    case GS_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case GS_ERROR_CAPACITY: return "capacity exceeded";
    case GS_ERROR_CUDA: return "CUDA error";
    case GS_ERROR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case GS_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case GS_ERROR_INTERNAL: return "device-side self-check failed";
  }
  return "unknown status";
}

uint32_t gs_version(void) { return kVersion; }

// ------------------------------------------------------------------ sorter

gs_status gs_sorter_create(gs_sorter** out) {
  if (!out) return GS_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  gs_sorter* s = new (std::nothrow) gs_sorter();
  if (!s) return GS_ERROR_OUT_OF_MEMORY;
  if (cudaGetDevice(&s->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess) {
    delete s;
    return GS_ERROR_CUDA;
  }
  if (cudaMalloc(&s->err, 256) != cudaSuccess) {
    delete s;
    return GS_ERROR_OUT_OF_MEMORY;
  }
  cudaMemset(s->err, 0, 256);
  *out = s;
  return GS_SUCCESS;
}

void gs_sorter_destroy(gs_sorter* s) {
  if (!s) return;
  cudaFree(s->err);
  delete s;
}

static size_t sorter_bytes(u32 max_count, size_t* status_off, size_t* alt_off) {
  const size_t control = align_up(kRadixControlBytes);
  const size_t status = align_up(radix_status_words(max_count) * sizeof(u64));
  const size_t alt = align_up((size_t)std::max(max_count, 1u) * sizeof(u32));
  if (status_off) *status_off = control;
  if (alt_off) *alt_off = control + status;
  return control + status + 2 * alt;
}

gs_status gs_sorter_key_value_storage_requirements(gs_sorter* s, uint32_t max_count, size_t* bytes) {
  if (!s || !bytes) return GS_ERROR_INVALID_ARGUMENT;
  *bytes = sorter_bytes(max_count, nullptr, nullptr);
  return GS_SUCCESS;
}

gs_status gs_sorter_sort_key_value_indirect(gs_sorter* s, gs_stream stream, uint32_t max_count, const uint32_t* count,
                                            uint32_t* keys, uint32_t* values, void* storage, size_t storage_bytes) {
  if (!s || !count || !keys || !values || !storage) return GS_ERROR_INVALID_ARGUMENT;
  size_t status_off = 0, alt_off = 0;
  const size_t need = sorter_bytes(max_count, &status_off, &alt_off);
  if (storage_bytes < need) return GS_ERROR_CAPACITY;
  if (max_count == 0) return GS_SUCCESS;
  char* base = static_cast<char*>(storage);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(base + status_off, 0, alt_off - status_off, st) != cudaSuccess) return GS_ERROR_CUDA;
  const size_t alt_words = align_up((size_t)max_count * sizeof(u32)) / sizeof(u32);
  RadixSortArgs a{};
  a.keys = keys;
  a.values = values;
  a.keys_alt = reinterpret_cast<u32*>(base + alt_off);
  a.values_alt = a.keys_alt + alt_words;
  a.count = count;
  a.max_count = max_count;
  a.begin_bit = 0;
  a.end_bit = 32;
  a.control = reinterpret_cast<u32*>(base);
  a.status = reinterpret_cast<u64*>(base + status_off);
  a.epoch = 1;
  a.err = s->err;
  a.num_sms = s->num_sms;
  return from_cuda(radix_sort(a, st));  // 4 passes: the result is back in keys/values
}

gs_status gs_sorter_check(gs_sorter* s, gs_stream stream) {
  if (!s) return GS_ERROR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return GS_ERROR_CUDA;
  u32 e = 0;
  if (cudaMemcpy(&e, s->err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return GS_ERROR_CUDA;
  cudaMemset(s->err, 0, 4);
  if (e & ERR_TIMEOUT) return GS_ERROR_DEVICE_TIMEOUT;
  if (e & ERR_INTERNAL) return GS_ERROR_INTERNAL;
  if (e & ERR_CAPACITY) return GS_ERROR_CAPACITY;
  return GS_SUCCESS;
}

// ------------------------------------------------------------------ context

static u32 default_pairs(const gs_context_options* o) {
  return o->max_tile_pairs ? o->max_tile_pairs : (u32)std::min<uint64_t>(16ull * o->max_splats, 0x3fffffffull);
}

gs_status gs_context_scratch_bytes(const gs_context_options* o, size_t* bytes) {
  if (!o || !bytes || o->max_width == 0 || o->max_height == 0) return GS_ERROR_INVALID_ARGUMENT;
  const u32 tiles_x = (o->max_width + kTile - 1) / kTile, tiles_y = (o->max_height + kTile - 1) / kTile;
  if ((uint64_t)tiles_x * tiles_y > kMaxTiles) return GS_ERROR_CAPACITY;
  Carver plan;
  gs_context probe;
  context_layout(plan, &probe, o->max_splats, o->max_width, o->max_height, default_pairs(o));
  *bytes = plan.offset;
  return GS_SUCCESS;
}

gs_status gs_context_create(gs_context** out, const gs_context_options* o) {
  if (!out || !o) return GS_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (o->max_width == 0 || o->max_height == 0) return GS_ERROR_INVALID_ARGUMENT;
  gs_context* c = new (std::nothrow) gs_context();
  if (!c) return GS_ERROR_OUT_OF_MEMORY;
  if (cudaGetDevice(&c->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      cull_stream_init() != cudaSuccess) {
    delete c;
    return GS_ERROR_CUDA;
  }
  const gs_status st = context_allocate(c, o->max_splats, o->max_width, o->max_height, default_pairs(o));
  if (st != GS_SUCCESS) {
    delete c;
    return st;
  }
  *out = c;
  return GS_SUCCESS;
}

static void destroy_lanes(gs_context* c) {
  if (c->nlanes) cudaDeviceSynchronize();
  for (u32 l = 0; l < c->nlanes; ++l) {
    gs_context_destroy(c->lane[l]);
    if (c->lane_join[l]) cudaEventDestroy(c->lane_join[l]);
    if (c->lane_stream[l]) cudaStreamDestroy(c->lane_stream[l]);
    c->lane[l] = nullptr;
    c->lane_join[l] = nullptr;
    c->lane_stream[l] = nullptr;
  }
  if (c->batch_fork) cudaEventDestroy(c->batch_fork);
  c->batch_fork = nullptr;
  for (cudaEvent_t& e : c->chunk_done) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  c->nlanes = 0;
}

static void free_batch_buffers(gs_context* c) {
  if (c->batch_arena) {
    cudaDeviceSynchronize();
    cudaFree(c->batch_arena);
    ++c->batch_gen;
  }
  c->batch_arena = nullptr;
  c->batch_bytes = 0;
  c->batch_views = c->batch_n = 0;
}

void gs_context_destroy(gs_context* c) {
  if (!c) return;
  destroy_lanes(c);
  free_batch_buffers(c);
  if (c->arena) {
    cudaDeviceSynchronize();
    cudaFree(c->arena);
  }
  if (c->events) {
    for (u32 i = 0; i < gs_context::kTimingRing * gs_context::kFrameEvents; ++i) cudaEventDestroy(c->events[i]);
    delete[] c->events;
  }
  delete c;
}

gs_status gs_context_enable_timing(gs_context* c, int enable) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  if (enable && !c->events) {
    const u32 total = gs_context::kTimingRing * gs_context::kFrameEvents;
    c->events = new (std::nothrow) cudaEvent_t[total];
    if (!c->events) return GS_ERROR_OUT_OF_MEMORY;
    for (u32 i = 0; i < total; ++i) {
      if (cudaEventCreate(&c->events[i]) != cudaSuccess) {
        for (u32 j = 0; j < i; ++j) cudaEventDestroy(c->events[j]);
        delete[] c->events;
        c->events = nullptr;
        return GS_ERROR_CUDA;
      }
    }
  }
  c->timing = enable != 0;
  c->timed_frames = 0;
  return GS_SUCCESS;
}

gs_status gs_context_stage_times(gs_context* c, uint32_t max_frames, float* ms, uint32_t* frames) {
  if (!c || !frames || (max_frames && !ms)) return GS_ERROR_INVALID_ARGUMENT;
  *frames = 0;
  if (!c->events || c->timed_frames == 0) return GS_SUCCESS;
  if (cudaDeviceSynchronize() != cudaSuccess) return GS_ERROR_CUDA;
  const u32 kept = std::min(c->timed_frames, gs_context::kTimingRing);
  const u32 rows = std::min(kept, max_frames);
  const u32 first = c->timed_frames - kept;
  for (u32 r = 0; r < rows; ++r) {
    cudaEvent_t* ev = c->frame_events(first + r);
    const u32 slabs = c->frame_slabs[(first + r) % gs_context::kTimingRing];
    float* row = ms + (size_t)r * GS_NUM_STAGES;
    for (int s = 0; s < GS_NUM_STAGES; ++s) row[s] = 0.0f;
    auto add = [&](int stage, int e0, int e1) {
      float t = 0.0f;
      if (cudaEventElapsedTime(&t, ev[e0], ev[e1]) != cudaSuccess) return false;
      row[stage] += t;
      return true;
    };
    if (!add(0, 0, 1) || !add(1, 1, 2)) return GS_ERROR_CUDA;
    for (u32 k = 0; k < slabs; ++k) {  // stages 2..5 summed over the slabs
      const int b = 3 + 4 * (int)k, prev = k ? b - 1 : 2;
      if (!add(2, prev, b) || !add(3, b, b + 1) || !add(4, b + 1, b + 2) || !add(5, b + 2, b + 3))
        return GS_ERROR_CUDA;
    }
  }
  *frames = rows;
  c->timed_frames = 0;
  return GS_SUCCESS;
}

gs_status gs_context_reserve(gs_context* c, const gs_context_options* o) {
  if (!c || !o) return GS_ERROR_INVALID_ARGUMENT;
  const u32 n = std::max(c->max_splats, o->max_splats);
  const u32 w = std::max(c->max_width, o->max_width), h = std::max(c->max_height, o->max_height);
  u32 pairs = std::max(c->pair_capacity, o->max_tile_pairs);
  if (pairs > 0x3fffffffu) return GS_ERROR_CAPACITY;
  for (u32 l = 0; l < c->nlanes; ++l) {
    const gs_status ls = gs_context_reserve(c->lane[l], o);
    if (ls != GS_SUCCESS) return ls;
  }
  if (n == c->max_splats && w == c->max_width && h == c->max_height && pairs == c->pair_capacity) return GS_SUCCESS;
  if (cudaDeviceSynchronize() != cudaSuccess) return GS_ERROR_CUDA;
  c->train_gen = 0;  // the differentiable forward's state lived in the old arena
  return context_allocate(c, n, w, h, pairs);
}

gs_status gs_context_set_slabs(gs_context* c, uint32_t count, const uint32_t* ends) {
  if (!c || !ends || count == 0 || count > GS_MAX_SLABS) return GS_ERROR_INVALID_ARGUMENT;
  for (u32 i = 0; i < count; ++i)
    if (ends[i] == 0 || ends[i] > 1024 || (i && ends[i] <= ends[i - 1])) return GS_ERROR_INVALID_ARGUMENT;
  if (ends[count - 1] != 1024) return GS_ERROR_INVALID_ARGUMENT;
  c->slab_count = count;
  for (u32 i = 0; i < GS_MAX_SLABS; ++i) c->slab_end[i] = i < count ? ends[i] : 1024;
  for (u32 l = 0; l < c->nlanes; ++l) gs_context_set_slabs(c->lane[l], count, ends);
  return GS_SUCCESS;
}

gs_status gs_context_set_train_slab_min(gs_context* c, uint32_t splats) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  c->train_slab_min = splats;
  for (u32 l = 0; l < c->nlanes; ++l) c->lane[l]->train_slab_min = splats;
  return GS_SUCCESS;
}

gs_status gs_context_set_cull_staging(gs_context* c, int enable) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  c->staged_cull = enable != 0;
  return GS_SUCCESS;
}

gs_status gs_context_set_lean(gs_context* c, int enable) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  c->lean = enable != 0;
  return GS_SUCCESS;
}

gs_status gs_context_set_transmittance_floor(gs_context* c, float t_floor) {
  if (!c || !(t_floor > 0.0f) || !(t_floor <= 1.0f / 255.0f)) return GS_ERROR_INVALID_ARGUMENT;
  c->t_floor = t_floor;
  for (u32 l = 0; l < c->nlanes; ++l) gs_context_set_transmittance_floor(c->lane[l], t_floor);
  return GS_SUCCESS;
}

gs_status gs_context_set_count_fragments(gs_context* c, int enable) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  c->count_fragments = enable ? 1 : 0;
  for (u32 l = 0; l < c->nlanes; ++l) gs_context_set_count_fragments(c->lane[l], enable);
  return GS_SUCCESS;
}

// Words of one slab's tile-range array at the context's capacity (tiles + 1 entries of 2 words).
static size_t range_words(const gs_context* c) { return (size_t)(c->max_tiles + 1) * 2; }

// A view culled and projected beforehand (k_cull_views): its compacted keys/ids, records, visible count.
struct PreCulled {
  u32* key;
  u32* index;
  float4* record;
  u32* visible;
};

// One frame.  sh32 (the differentiable path): FP32 SH instead of s->sh, every slab's tile lists kept
// (stacked), and the training raster that stores per-pixel blend counts and final transmittance.  pre: the cull already
// ran for this view (the batched form); the frame starts at the depth sort on pre's buffers.
static gs_status render_frame(gs_context* c, const gs_splats* s, const float* sh32, const gs_camera* cam,
                              const gs_target* t, const gs_frame_outputs* outs, gs_stream stream,
                              const PreCulled* pre = nullptr) {
  const bool train = sh32 != nullptr;
  gs_frame_outputs none{};
  const gs_frame_outputs& o = outs ? *outs : none;
  c->last_batched = false;
  c->train_gen = train ? ++c->frame_gen : (++c->frame_gen, 0);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const u32 n = s->count;
  const u32 W = cam->width, H = cam->height;
  const u32 tiles_x = (W + kTile - 1) / kTile, tiles_y = (H + kTile - 1) / kTile;
  const u32 tiles = tiles_x * tiles_y;

  FrameConst fc;
  frame_constants(cam->projection, cam->view, cam->model, cam->camera_position, W, H, n, &fc);

#define GS_TRY(x)                                  \
  do {                                             \
    if ((x) != cudaSuccess) return GS_ERROR_CUDA; \
  } while (0)

  cudaEvent_t* ev = c->timing ? c->frame_events(c->timed_frames++) : nullptr;
#define GS_MARK(i) \
  if (ev) GS_TRY(cudaEventRecord(ev[i], st))
  GS_MARK(0);
  GS_TRY(cudaMemsetAsync(c->frame, 0, FW_WORDS * sizeof(u32), st));
  // Look-back status words are cleared every frame and the frame's waits use fixed epochs (1: cull,
  // 2-5: depth sort passes), so a frame captured in a CUDA graph replays correctly.
  GS_TRY(cudaMemsetAsync(c->arena + c->status_bytes_begin, 0, c->status_bytes_end - c->status_bytes_begin, st));
  GS_TRY(cudaMemsetAsync(c->tile_done, 0, (size_t)(tiles + 31) / 32 * sizeof(u32), st));
  u32* key = pre ? pre->key : (o.keys ? o.keys : c->key);
  u32* index = pre ? pre->index : (o.index ? o.index : c->index);
  float4* record = pre ? pre->record : c->record;
  u32* visible = c->frame + FW_VISIBLE;
  if (pre) GS_TRY(cudaMemcpyAsync(visible, pre->visible, sizeof(u32), cudaMemcpyDeviceToDevice, st));
  const bool want_inst = o.instances != nullptr;

  CullArgs ca{};
  ca.position = s->position;
  ca.cov3d = s->cov3d;
  ca.opacity = s->opacity;
  ca.sh = s->sh;
  ca.sh32 = sh32;
  ca.key = key;
  ca.index = index;
  ca.record = record;
  ca.inst_by_id = want_inst ? c->inst_by_id : nullptr;
  ca.visible_count = visible;
  ca.status = c->cull_status;
  ca.ticket = c->frame + FW_TICKET_CULL;
  ca.epoch = 1;
  ca.err = c->err;
  ca.num_sms = c->num_sms;
  ca.staged = c->staged_cull ? 1 : 0;
  ca.lean = c->lean ? 1 : 0;
  if (!pre) GS_TRY(launch_cull_project(fc, ca, st));
  GS_MARK(1);

  if (n > 0) {
    RadixSortArgs ra{};
    ra.keys = key;
    ra.values = index;
    ra.keys_alt = c->key_alt;
    ra.values_alt = c->index_alt;
    ra.count = visible;
    ra.max_count = n;
    ra.begin_bit = 0;
    ra.end_bit = 32;
    ra.control = c->radix_control;
    ra.status = c->radix_status;
    ra.epoch = 2;
    ra.err = c->err;
    ra.num_sms = c->num_sms;
    ra.lean = c->lean ? 1 : 0;
    GS_TRY(radix_sort(ra, st));  // 4 passes: sorted keys/index are back in key/index
  }

  if (want_inst || o.draw_indirect)
    GS_TRY(launch_instances(index, visible, c->inst_by_id, n, o.instances, o.draw_indirect, st));
  GS_MARK(2);

  // Depth slabs, nearest first (one slab when nothing is visible).  The differentiable forward keeps
  // every slab's tile lists (stacked in the pair arrays, a tile-range array per slab) and blended
  // counts for its backward.
  const u32 slabs = (n > 0 && (!train || n >= c->train_slab_min)) ? c->slab_count : 1;
  const size_t range_stride = range_words(c);
  const size_t pix_stride = (size_t)c->max_width * c->max_height;
  if (train) {
    c->train_slabs = slabs;
    c->train_record = record;
    for (u32 k = 1; k < slabs; ++k)  // tiles finished earlier are skipped by later slabs: count 0
      GS_TRY(cudaMemsetAsync(c->train_nproc + k * pix_stride, 0, (size_t)W * H * sizeof(u32), st));
  }
  if (ev) c->frame_slabs[(c->timed_frames - 1) % gs_context::kTimingRing] = slabs;
  for (u32 k = 0; k < slabs; ++k) {
    const int e = 3 + 4 * (int)k;
    BinArgs ba{};
    ba.index = index;
    ba.visible_count = visible;
    ba.record = record;
    ba.n = n;
    ba.slab_e0 = k ? c->slab_end[k - 1] : 0;
    ba.slab_e1 = slabs == 1 ? 1024 : c->slab_end[k];
    ba.tile_done = k ? c->tile_done : nullptr;
    ba.width = W;
    ba.height = H;
    ba.tiles_x = tiles_x;
    ba.tiles_y = tiles_y;
    ba.count = c->bin_count;
    ba.diff = c->bin_diff;
    ba.tile_range = train ? c->tile_range + k * range_stride : c->tile_range;
    ba.stack_slabs = train;
    ba.tile_order = c->tile_order;
    ba.giant_list = c->giant_list;
    ba.giant_count = c->frame + FW_GIANTS + k;
    ba.pair_key = c->pair_key;
    ba.pair_splat = c->pair_splat;
    ba.pair_capacity = c->pair_capacity;
    ba.slab_pairs = c->frame + FW_SLAB_PAIRS;
    ba.pair_total = c->frame + FW_PAIR_TOTAL;
    ba.pair_sum = reinterpret_cast<unsigned long long*>(c->frame + FW_PAIR_SUM);
    ba.pair_peak = c->err + 1;
    ba.err = c->err;
    ba.lean = c->lean ? 1 : 0;
    GS_TRY(launch_bin(ba, st, ev ? ev[e] : nullptr, ev ? ev[e + 1] : nullptr, c->num_sms));
    GS_MARK(e + 2);

    RasterArgs rr{};
    rr.tile_range = ba.tile_range;
    rr.pair_capacity = c->pair_capacity;
    rr.pair_splat = c->pair_splat;
    rr.record = record;
    rr.width = W;
    rr.height = H;
    rr.tiles_x = tiles_x;
    rr.tiles_y = tiles_y;
    rr.out_rgba = t->color_rgba32f;
    rr.out_bgra = reinterpret_cast<uchar4*>(t->color_bgra8);
    rr.depth = t->depth;
    rr.t_floor = c->t_floor;
    rr.fragments = c->count_fragments ? reinterpret_cast<unsigned long long*>(c->frame + FW_FRAGMENTS) : nullptr;
    rr.state_c = c->state_c;
    rr.state_t = c->state_t;
    rr.tile_done = c->tile_done;
    rr.first = k == 0;
    rr.last = k + 1 == slabs;
    rr.nproc = train ? c->train_nproc + k * pix_stride : nullptr;
    rr.lean = c->lean ? 1 : 0;
    GS_TRY(launch_raster(rr, st));
    GS_MARK(e + 3);
  }

  if (o.visible_count)
    GS_TRY(cudaMemcpyAsync(o.visible_count, visible, sizeof(u32), cudaMemcpyDeviceToDevice, st));
#undef GS_MARK
#undef GS_TRY
  return GS_SUCCESS;
}

gs_status gs_render(gs_context* c, const gs_splats* s, const gs_camera* cam, const gs_target* t,
                    const gs_frame_outputs* outs, gs_stream stream) {
  if (!c || !s || !cam || !t) return GS_ERROR_INVALID_ARGUMENT;
  if (!t->color_rgba32f && !t->color_bgra8) return GS_ERROR_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return GS_ERROR_INVALID_ARGUMENT;
  if (s->count && (!s->position || !s->cov3d || !s->opacity || !s->sh)) return GS_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(s->sh) & 15u) != 0) return GS_ERROR_INVALID_ARGUMENT;
  if (s->count > c->max_splats || cam->width > c->max_width || cam->height > c->max_height) return GS_ERROR_CAPACITY;
  if (s->count > 0x3fffffffu) return GS_ERROR_CAPACITY;
  return render_frame(c, s, nullptr, cam, t, outs, stream);
}

static gs_status check_train_params(const gs_context* c, const gs_train_params* p, const gs_camera* cam) {
  if (!p || !cam) return GS_ERROR_INVALID_ARGUMENT;
  if (cam->width == 0 || cam->height == 0) return GS_ERROR_INVALID_ARGUMENT;
  if (p->count && (!p->means || !p->log_scales || !p->quats || !p->opacity_logits || !p->sh))
    return GS_ERROR_INVALID_ARGUMENT;
  if (((reinterpret_cast<uintptr_t>(p->quats) | reinterpret_cast<uintptr_t>(p->sh)) & 15u) != 0)
    return GS_ERROR_INVALID_ARGUMENT;
  if (p->count > c->max_splats || cam->width > c->max_width || cam->height > c->max_height) return GS_ERROR_CAPACITY;
  return GS_SUCCESS;
}

gs_status gs_train_forward(gs_context* c, const gs_train_params* p, const gs_camera* cam, float* color,
                           gs_stream stream) {
  if (!c || !color) return GS_ERROR_INVALID_ARGUMENT;
  const gs_status v = check_train_params(c, p, cam);
  if (v != GS_SUCCESS) return v;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  TrainArgs ta{};
  ta.means = p->means;
  ta.log_scales = p->log_scales;
  ta.quats = p->quats;
  ta.opacity_logits = p->opacity_logits;
  ta.sh = p->sh;
  ta.n = p->count;
  ta.position = c->train_pos;
  ta.cov3d = c->train_cov;
  ta.opacity = c->train_opacity;
  if (launch_activate(ta, st) != cudaSuccess) return GS_ERROR_CUDA;
  gs_splats s{c->train_pos, c->train_cov, c->train_opacity, nullptr, p->count};
  gs_target t{color, nullptr, nullptr};
  return render_frame(c, &s, p->sh, cam, &t, nullptr, stream);
}

static gs_status check_train_grads(const gs_train_params* p, const gs_train_grads* g) {
  if (!g) return GS_ERROR_INVALID_ARGUMENT;
  if (p->count && (!g->means || !g->log_scales || !g->quats || !g->opacity_logits || !g->sh))
    return GS_ERROR_INVALID_ARGUMENT;
  if (((reinterpret_cast<uintptr_t>(g->quats) | reinterpret_cast<uintptr_t>(g->sh)) & 15u) != 0)
    return GS_ERROR_INVALID_ARGUMENT;
  return GS_SUCCESS;
}

// The backward of the last differentiable forward held by context c (one view).
// The blend backward of the last differentiable forward held by context c: fills c->grad_rec.
static gs_status blend_backward(gs_context* c, const gs_train_params* p, const gs_camera* cam, const float* grad_rgba,
                                cudaStream_t st) {
  const u32 W = cam->width, H = cam->height;
  if (cudaMemsetAsync(c->grad_rec, 0, (size_t)p->count * kGradRec * sizeof(float), st) != cudaSuccess)
    return GS_ERROR_CUDA;
  RasterBackwardArgs rb{};
  rb.tile_range = c->tile_range;
  rb.range_stride = (u32)range_words(c);
  rb.slabs = c->train_slabs;
  rb.nproc_stride = c->max_width * c->max_height;
  rb.pair_capacity = c->pair_capacity;
  rb.pair_splat = c->pair_splat;
  rb.record = c->train_record ? c->train_record : c->record;
  rb.width = W;
  rb.height = H;
  rb.tiles_x = (W + kTile - 1) / kTile;
  rb.tiles_y = (H + kTile - 1) / kTile;
  rb.state_t = c->state_t;
  rb.nproc = c->train_nproc;
  rb.grad_rgba = reinterpret_cast<const float4*>(grad_rgba);
  rb.grad_rec = c->grad_rec;
  return from_cuda(launch_raster_backward(rb, st));
}

static_assert(kMaxTrainViews >= GS_MAX_LANES, "one projection backward covers every lane's view");

// The projection backward of n views at once; view v's blend gradients are in ctx[v]->grad_rec.
static gs_status project_backward(gs_context* const* ctx, const gs_camera* cams, u32 n, const gs_train_params* p,
                                  const gs_train_grads* g, cudaStream_t st) {
  std::unique_ptr<TrainViews> tv(new TrainViews{});
  tv->count = n;
  for (u32 v = 0; v < n; ++v) {
    const gs_camera& cam = cams[v];
    frame_constants(cam.projection, cam.view, cam.model, cam.camera_position, cam.width, cam.height, p->count,
                    &tv->fc[v]);
    tv->grad_rec[v] = ctx[v]->grad_rec;
    for (int r = 0; r < 4; ++r)  // column-major inputs: element (r, c) of a matrix m is m[4 c + r]
      for (int c = 0; c < 4; ++c) {
        double acc = 0.0;
        for (int k = 0; k < 4; ++k) acc += (double)cam.view[4 * k + r] * (double)cam.model[4 * c + k];
        tv->vm[v][4 * r + c] = (float)acc;
      }
  }
  TrainArgs ta{};
  ta.means = p->means;
  ta.log_scales = p->log_scales;
  ta.quats = p->quats;
  ta.opacity_logits = p->opacity_logits;
  ta.sh = p->sh;
  ta.n = p->count;
  ta.g_means = g->means;
  ta.g_log_scales = g->log_scales;
  ta.g_quats = g->quats;
  ta.g_opacity_logits = g->opacity_logits;
  ta.g_sh = g->sh;
  return from_cuda(launch_project_backward(*tv, ta, st));
}

gs_status gs_train_backward(gs_context* c, const gs_train_params* p, const gs_camera* cam, const float* grad_rgba,
                            const gs_train_grads* g, gs_stream stream) {
  if (!c || !grad_rgba) return GS_ERROR_INVALID_ARGUMENT;
  gs_status v = check_train_params(c, p, cam);
  if (v == GS_SUCCESS) v = check_train_grads(p, g);
  if (v != GS_SUCCESS) return v;
  if (c->train_gen == 0 || c->train_gen != c->frame_gen) return GS_ERROR_INVALID_ARGUMENT;  // state overwritten
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if ((v = blend_backward(c, p, cam, grad_rgba, st)) != GS_SUCCESS) return v;
  return project_backward(&c, cam, 1, p, g, st);
}

// Batched differentiable path: view v is drawn by render lane v, which keeps that view's forward state
// for the backward; the lanes' blend backwards run concurrently, then one projection backward adds the
// gradients of all views into the caller's buffers.
static gs_status fork_lanes(gs_context* c, u32 used, cudaStream_t st) {
  if (cudaEventRecord(c->batch_fork, st) != cudaSuccess) return GS_ERROR_CUDA;
  for (u32 l = 0; l < used; ++l)
    if (cudaStreamWaitEvent(c->lane_stream[l], c->batch_fork, 0) != cudaSuccess) return GS_ERROR_CUDA;
  return GS_SUCCESS;
}

static gs_status join_lanes(gs_context* c, u32 used, cudaStream_t st) {
  for (u32 l = 0; l < used; ++l) {
    if (cudaEventRecord(c->lane_join[l], c->lane_stream[l]) != cudaSuccess) return GS_ERROR_CUDA;
    if (cudaStreamWaitEvent(st, c->lane_join[l], 0) != cudaSuccess) return GS_ERROR_CUDA;
  }
  return GS_SUCCESS;
}

// Per-view cull outputs of the batched forms, for up to kMaxBatchViews views of up to max_splats
// splats: [visible words][tickets][look-back status of every view] (cleared per batch), then per view
// its compacted keys, ids and records.  Allocated by the first batched call that needs them (never
// while the stream is being captured: that call takes the per-lane cull instead).
constexpr u32 kMaxBatchViews = 64;
constexpr u32 kCullChunk = 8;  // views per shared-cull launch of the batched render (pipelined with the lanes)
static_assert(kMaxBatchViews / kCullChunk <= 64 && kCullChunk <= kMaxCullViews, "chunk events and launches");

struct BatchLayout {
  size_t status_off, head_bytes, status_words, view_stride, key_off, index_off, record_off, total;
};

static BatchLayout batch_layout(u32 views, u32 n) {
  BatchLayout b{};
  const auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  b.status_words = (n + kCullTile - 1) / kCullTile;
  b.status_off = up((size_t)(2 * kMaxBatchViews + 1) * sizeof(u32));  // visible words, tickets
  b.head_bytes = b.status_off + up((size_t)views * b.status_words * sizeof(u64));
  b.key_off = 0;
  b.index_off = up((size_t)n * sizeof(u32));
  b.record_off = b.index_off + up((size_t)n * sizeof(u32));
  b.view_stride = b.record_off + up((size_t)n * 4 * sizeof(float4));
  b.total = b.head_bytes + (size_t)views * b.view_stride;
  return b;
}

static bool batch_buffers(gs_context* c, u32 views, cudaStream_t st) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return false;
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  if (c->batch_arena && views <= c->batch_views && c->max_splats <= c->batch_n) {
    c->batch_captured |= capturing;
    return true;
  }
  // Growing frees the arena.  Never while capturing, and never once a capture has recorded the arena's
  // addresses: a graph holding them would replay into freed memory.  Those calls cull per lane instead.
  if (capturing || c->batch_captured) return false;
  free_batch_buffers(c);
  const BatchLayout b = batch_layout(views, c->max_splats);
  if (cudaMalloc(&c->batch_arena, b.total) != cudaSuccess) {
    cudaGetLastError();
    c->batch_arena = nullptr;
    return false;
  }
  c->batch_bytes = b.total;
  c->batch_views = views;
  c->batch_n = c->max_splats;
  return true;
}

// The arena's buffers of slot w.
static PreCulled batch_slot(const gs_context* c, u32 w) {
  const BatchLayout b = batch_layout(c->batch_views, c->batch_n);
  char* vb = c->batch_arena + b.head_bytes + (size_t)w * b.view_stride;
  return PreCulled{reinterpret_cast<u32*>(vb + b.key_off), reinterpret_cast<u32*>(vb + b.index_off),
                   reinterpret_cast<float4*>(vb + b.record_off), reinterpret_cast<u32*>(c->batch_arena) + w};
}

// The cull + projection of cams[0 .. nv) (nv <= batch_views) into arena slots 0 .. nv-1, k_cull_views
// launches of up to kMaxCullViews views on `st`.  sh32: FP32 SH (the differentiable path).
// Clears the arena's head (visible words, tickets, look-back status) before a batch's culls.
static gs_status batch_head_clear(gs_context* c, cudaStream_t st) {
  const BatchLayout b = batch_layout(c->batch_views, c->batch_n);
  ++c->batch_gen;
  return cudaMemsetAsync(c->batch_arena, 0, b.head_bytes, st) == cudaSuccess ? GS_SUCCESS : GS_ERROR_CUDA;
}

// One k_cull_views launch (cnt <= kMaxCullViews views) into arena slots slots[0 .. cnt), cams[slot] being
// the slot's camera, with launch ticket `ticket` of the batch.  sh32: FP32 SH (the differentiable path).
static gs_status cull_views_launch(gs_context* c, const gs_splats* s, const float* sh32, const u32* slots, u32 cnt,
                                   const gs_camera* cams, u32 ticket, cudaStream_t st) {
  const BatchLayout b = batch_layout(c->batch_views, c->batch_n);
  char* base = c->batch_arena;
  u32* tickets = reinterpret_cast<u32*>(base) + kMaxBatchViews;
  u64* status = reinterpret_cast<u64*>(base + b.status_off);
  std::unique_ptr<CullViewsArgs> ca(new CullViewsArgs{});
  ca->position = s->position;
  ca->cov3d = s->cov3d;
  ca->opacity = s->opacity;
  ca->sh = s->sh;
  ca->sh32 = sh32;
  ca->n = s->count;
  ca->count = cnt;
  ca->ticket = tickets + ticket;
  ca->epoch = 1;
  ca->err = c->err;
  ca->num_sms = c->num_sms;
  for (u32 i = 0; i < cnt; ++i) {
    const u32 w = slots[i];
    const gs_camera& cam = cams[w];
    frame_constants(cam.projection, cam.view, cam.model, cam.camera_position, cam.width, cam.height, s->count,
                    &ca->fc[i]);
    const PreCulled pre = batch_slot(c, w);
    ca->view[i] = CullView{pre.key, pre.index, pre.record, pre.visible, status + (size_t)w * b.status_words};
  }
  return launch_cull_views(*ca, st) == cudaSuccess ? GS_SUCCESS : GS_ERROR_CUDA;
}

// The cull + projection of cams[0 .. nv) (nv <= batch_views) into arena slots 0 .. nv-1, k_cull_views
// launches of up to kMaxCullViews views on `st`.  sh32: FP32 SH (the differentiable path).
static gs_status shared_cull(gs_context* c, const gs_splats* s, const float* sh32, u32 nv, const gs_camera* cams,
                             cudaStream_t st) {
  gs_status r = batch_head_clear(c, st);
  u32 slots[kMaxCullViews];
  for (u32 c0 = 0; r == GS_SUCCESS && c0 < nv; c0 += kMaxCullViews) {
    const u32 cnt = std::min(kMaxCullViews, nv - c0);
    for (u32 i = 0; i < cnt; ++i) slots[i] = c0 + i;
    r = cull_views_launch(c, s, sh32, slots, cnt, cams, c0 / kMaxCullViews, st);
  }
  return r;
}

// Views [v0, v0 + nv) of the batch: their culls in k_cull_views launches on `st`, then their frames
// from the depth sort on, spread over the lanes.
static gs_status batched_group(gs_context* c, const gs_splats* s, u32 v0, u32 nv, const gs_camera* cams,
                               const gs_target* targets, cudaStream_t st) {
  // Largest views first, each to the lane with the least work so far (work ~ pixels + a fixed cost per
  // view), so the lanes finish together.  The views are culled in chunks of kCullChunk in that order,
  // each chunk one k_cull_views launch on `st` followed by an event: a lane starts a view as soon as
  // its chunk is culled, so the later chunks' culls overlap the lanes' sorting, binning and blending.
  std::vector<u32> order(nv);
  for (u32 w = 0; w < nv; ++w) order[w] = w;
  const auto work = [&](u32 w) { return (double)cams[v0 + w].width * cams[v0 + w].height + 250000.0; };
  std::stable_sort(order.begin(), order.end(), [&](u32 x, u32 y) { return work(x) > work(y); });
  gs_status r = batch_head_clear(c, st);
  if (r != GS_SUCCESS) return r;
  const u32 used = std::min(c->nlanes, std::max(nv, 1u));
  double load[GS_MAX_LANES] = {};
  bool forked[GS_MAX_LANES] = {};
  for (u32 k0 = 0, chunk = 0; k0 < nv; k0 += kCullChunk, ++chunk) {
    const u32 cnt = std::min(kCullChunk, nv - k0);
    if ((r = cull_views_launch(c, s, nullptr, order.data() + k0, cnt, cams + v0, chunk, st)) != GS_SUCCESS) return r;
    if (cudaEventRecord(c->chunk_done[chunk], st) != cudaSuccess) return GS_ERROR_CUDA;
    for (u32 i = 0; i < cnt; ++i) {
      const u32 w = order[k0 + i];
      u32 l = 0;
      for (u32 k = 1; k < used; ++k)
        if (load[k] < load[l]) l = k;
      load[l] += work(w);
      if (cudaStreamWaitEvent(c->lane_stream[l], c->chunk_done[chunk], 0) != cudaSuccess) return GS_ERROR_CUDA;
      forked[l] = true;
      const PreCulled pre = batch_slot(c, w);
      r = render_frame(c->lane[l], s, nullptr, &cams[v0 + w], &targets[v0 + w], nullptr,
                       reinterpret_cast<gs_stream>(c->lane_stream[l]), &pre);
      if (r != GS_SUCCESS) return r;
    }
  }
  for (u32 l = 0; l < used; ++l) {  // join the lanes that took views
    if (!forked[l]) continue;
    if (cudaEventRecord(c->lane_join[l], c->lane_stream[l]) != cudaSuccess) return GS_ERROR_CUDA;
    if (cudaStreamWaitEvent(st, c->lane_join[l], 0) != cudaSuccess) return GS_ERROR_CUDA;
  }
  return GS_SUCCESS;
}


gs_status gs_train_forward_batched(gs_context* c, const gs_train_params* p, uint32_t n_views, const gs_camera* cams,
                                   float* const* colors, gs_stream stream) {
  if (!c || (n_views && (!cams || !colors))) return GS_ERROR_INVALID_ARGUMENT;
  if (n_views > c->nlanes) return GS_ERROR_CAPACITY;  // one lane per view holds its forward state
  for (u32 v = 0; v < n_views; ++v) {
    const gs_status r = check_train_params(c, p, &cams[v]);
    if (r != GS_SUCCESS) return r;
    if (!colors[v]) return GS_ERROR_INVALID_ARGUMENT;
  }
  if (n_views == 0) return GS_SUCCESS;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  TrainArgs ta{};  // the activation once, shared by every view
  ta.means = p->means;
  ta.log_scales = p->log_scales;
  ta.quats = p->quats;
  ta.opacity_logits = p->opacity_logits;
  ta.sh = p->sh;
  ta.n = p->count;
  ta.position = c->train_pos;
  ta.cov3d = c->train_cov;
  ta.opacity = c->train_opacity;
  if (launch_activate(ta, st) != cudaSuccess) return GS_ERROR_CUDA;
  const gs_splats s{c->train_pos, c->train_cov, c->train_opacity, nullptr, p->count};
  // one shared cull + projection pass for all views when its buffers are available (each lane then
  // starts at the depth sort and keeps pointing at its view's records for the backward)
  const bool shared = p->count > 0 && c->multi_view_cull && batch_buffers(c, n_views, st);
  gs_status r = shared ? shared_cull(c, &s, p->sh, n_views, cams, st) : GS_SUCCESS;
  if (r != GS_SUCCESS) return r;
  if ((r = fork_lanes(c, n_views, st)) != GS_SUCCESS) return r;
  for (u32 v = 0; v < n_views; ++v) {
    gs_target t{colors[v], nullptr, nullptr};
    const PreCulled pre = shared ? batch_slot(c, v) : PreCulled{};
    r = render_frame(c->lane[v], &s, p->sh, &cams[v], &t, nullptr, reinterpret_cast<gs_stream>(c->lane_stream[v]),
                     shared ? &pre : nullptr);
    if (r != GS_SUCCESS) return r;
  }
  c->last_batched = true;
  c->train_batch_gen = shared ? c->batch_gen : 0;
  c->train_views = n_views;
  return join_lanes(c, n_views, st);
}

gs_status gs_train_backward_batched(gs_context* c, const gs_train_params* p, uint32_t n_views, const gs_camera* cams,
                                    const float* const* grads_rgba, const gs_train_grads* g, gs_stream stream) {
  if (!c || (n_views && (!cams || !grads_rgba))) return GS_ERROR_INVALID_ARGUMENT;
  if (n_views > c->nlanes) return GS_ERROR_CAPACITY;
  for (u32 v = 0; v < n_views; ++v) {
    const gs_status r = check_train_params(c, p, &cams[v]);
    if (r != GS_SUCCESS) return r;
    if (!grads_rgba[v]) return GS_ERROR_INVALID_ARGUMENT;
  }
  gs_status r = check_train_grads(p, g);
  if (r != GS_SUCCESS || n_views == 0) return r;
  // the forward state of every view must still be the last batched differentiable forward's: its
  // lanes' lists and, with the shared cull, its records in the batch arena
  if (n_views != c->train_views) return GS_ERROR_INVALID_ARGUMENT;
  if (c->train_batch_gen != 0 && c->train_batch_gen != c->batch_gen) return GS_ERROR_INVALID_ARGUMENT;
  for (u32 v = 0; v < n_views; ++v)
    if (c->lane[v]->train_gen == 0 || c->lane[v]->train_gen != c->lane[v]->frame_gen) return GS_ERROR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if ((r = fork_lanes(c, n_views, st)) != GS_SUCCESS) return r;
  for (u32 v = 0; v < n_views; ++v) {  // the views' blend backwards run concurrently
    r = blend_backward(c->lane[v], p, &cams[v], grads_rgba[v], c->lane_stream[v]);
    if (r != GS_SUCCESS) return r;
  }
  if ((r = join_lanes(c, n_views, st)) != GS_SUCCESS) return r;
  return project_backward(c->lane, cams, n_views, p, g, st);  // then one pass over the splats for all views
}

// ------------------------------------------------------------------ viewer loop (CUDA graph per frame)

// One captured frame of the viewer: its context (the caller's for slot 0, an own one otherwise), the
// graph and the cull node whose camera constants are rewritten per frame.
struct ViewerSlot {
  gs_context* ctx = nullptr;
  bool own_ctx = false;
  cudaStream_t stream = nullptr;  // capture stream; with frames in flight also the slot's launch stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t cull = nullptr;
  CullArgs cull_args{};
  cudaKernelNodeParams cull_params{};
  cudaEvent_t done = nullptr;
};

struct gs_viewer {
  u32 nslots = 0;
  ViewerSlot slot[GS_MAX_FRAMES_IN_FLIGHT];
  cudaEvent_t fork = nullptr;
  u32 next = 0;  // slot of the next frame
  u32 width = 0, height = 0, count = 0;
};

void gs_viewer_destroy(gs_viewer* v) {
  if (!v) return;
  if (v->nslots > 1) cudaDeviceSynchronize();
  for (u32 i = 0; i < v->nslots; ++i) {
    ViewerSlot& sl = v->slot[i];
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.graph) cudaGraphDestroy(sl.graph);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.own_ctx) gs_context_destroy(sl.ctx);
  }
  if (v->fork) cudaEventDestroy(v->fork);
  delete v;
}

static gs_status capture_slot(ViewerSlot& sl, const gs_splats* s, const gs_camera* cam, const gs_target* t) {
  if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) return GS_ERROR_CUDA;
  if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) return GS_ERROR_CUDA;
  if (cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GS_ERROR_CUDA;
  const gs_status r = gs_render(sl.ctx, s, cam, t, nullptr, reinterpret_cast<gs_stream>(sl.stream));
  const cudaError_t e = cudaStreamEndCapture(sl.stream, &sl.graph);
  if (r != GS_SUCCESS) return r;
  if (e != cudaSuccess) return GS_ERROR_CUDA;
  size_t count = 0;
  if (cudaGraphGetNodes(sl.graph, nullptr, &count) != cudaSuccess) return GS_ERROR_CUDA;
  std::vector<cudaGraphNode_t> nodes(count);
  if (count && cudaGraphGetNodes(sl.graph, nodes.data(), &count) != cudaSuccess) return GS_ERROR_CUDA;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType type;
    if (cudaGraphNodeGetType(node, &type) != cudaSuccess || type != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams kp{};
    if (cudaGraphKernelNodeGetParams(node, &kp) != cudaSuccess) continue;
    if (!is_cull_kernel(kp.func)) continue;
    sl.cull = node;
    sl.cull_params = kp;
    sl.cull_args = *reinterpret_cast<const CullArgs*>(kp.kernelParams[1]);
  }
  if (s->count && !sl.cull) return GS_ERROR_INTERNAL;
  if (cudaGraphInstantiate(&sl.exec, sl.graph, 0) != cudaSuccess) return GS_ERROR_CUDA;
  return GS_SUCCESS;
}

gs_status gs_viewer_create_frames(gs_viewer** out, gs_context* c, const gs_splats* s, const gs_camera* cam,
                                  const gs_target* targets, uint32_t frames_in_flight) {
  if (!out || !c || !s || !cam || !targets) return GS_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (frames_in_flight == 0 || frames_in_flight > GS_MAX_FRAMES_IN_FLIGHT || c->timing) return GS_ERROR_INVALID_ARGUMENT;
  gs_viewer* v = new (std::nothrow) gs_viewer();
  if (!v) return GS_ERROR_OUT_OF_MEMORY;
  v->width = cam->width;
  v->height = cam->height;
  v->count = s->count;
  const auto fail = [&](gs_status st) {
    gs_viewer_destroy(v);
    return st;
  };
  if (cudaEventCreateWithFlags(&v->fork, cudaEventDisableTiming) != cudaSuccess) return fail(GS_ERROR_CUDA);
  gs_context_options o{c->max_splats, c->max_width, c->max_height, c->pair_capacity};
  for (u32 i = 0; i < frames_in_flight; ++i) {
    ViewerSlot& sl = v->slot[i];
    v->nslots = i + 1;  // what exists so far is torn down on failure
    if (i == 0) {
      sl.ctx = c;
    } else {  // an own context with the caller's settings
      gs_status st = gs_context_create(&sl.ctx, &o);
      if (st != GS_SUCCESS) return fail(st);
      sl.own_ctx = true;
      gs_context_set_slabs(sl.ctx, c->slab_count, c->slab_end);
      gs_context_set_count_fragments(sl.ctx, c->count_fragments);
      gs_context_set_transmittance_floor(sl.ctx, c->t_floor);
      gs_context_set_cull_staging(sl.ctx, c->staged_cull);
    }
    // With frames in flight every slot's frames run beside the others': capture them lean (the
    // caller's own setting is restored afterwards; captured launches keep their configuration).
    const bool lean = sl.ctx->lean;
    sl.ctx->lean = lean || frames_in_flight > 1;
    const gs_status st = capture_slot(sl, s, cam, &targets[i]);
    sl.ctx->lean = lean;
    if (st != GS_SUCCESS) return fail(st);
  }
  *out = v;
  return GS_SUCCESS;
}

gs_status gs_viewer_create(gs_viewer** out, gs_context* c, const gs_splats* s, const gs_camera* cam,
                           const gs_target* t) {
  return gs_viewer_create_frames(out, c, s, cam, t, 1);
}

gs_status gs_viewer_submit(gs_viewer* v, const gs_camera* cam, gs_stream stream, uint32_t* slot_out) {
  if (!v || !cam) return GS_ERROR_INVALID_ARGUMENT;
  if (cam->width != v->width || cam->height != v->height) return GS_ERROR_INVALID_ARGUMENT;
  const u32 i = v->next;
  ViewerSlot& sl = v->slot[i];
  if (sl.cull) {  // later launches of the graph see the new camera; launches in flight keep theirs
    FrameConst fc;
    frame_constants(cam->projection, cam->view, cam->model, cam->camera_position, v->width, v->height, v->count, &fc);
    CullArgs ca = sl.cull_args;
    void* args[2] = {&fc, &ca};
    cudaKernelNodeParams kp = sl.cull_params;
    kp.kernelParams = args;
    kp.extra = nullptr;
    if (cudaGraphExecKernelNodeSetParams(sl.exec, sl.cull, &kp) != cudaSuccess) return GS_ERROR_CUDA;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (v->nslots == 1) {  // one slot: the frame runs on the caller's stream
    if (cudaGraphLaunch(sl.exec, st) != cudaSuccess || cudaEventRecord(sl.done, st) != cudaSuccess)
      return GS_ERROR_CUDA;
  } else {  // after the caller's prior work, on the slot's stream (its previous frame precedes it there)
    if (cudaEventRecord(v->fork, st) != cudaSuccess || cudaStreamWaitEvent(sl.stream, v->fork, 0) != cudaSuccess ||
        cudaGraphLaunch(sl.exec, sl.stream) != cudaSuccess || cudaEventRecord(sl.done, sl.stream) != cudaSuccess)
      return GS_ERROR_CUDA;
  }
  if (slot_out) *slot_out = i;
  v->next = (i + 1) % v->nslots;
  return GS_SUCCESS;
}

gs_status gs_viewer_wait(gs_viewer* v, uint32_t slot, gs_stream stream) {
  if (!v || slot >= v->nslots) return GS_ERROR_INVALID_ARGUMENT;
  return from_cuda(cudaStreamWaitEvent(reinterpret_cast<cudaStream_t>(stream), v->slot[slot].done, 0));
}

gs_status gs_viewer_frame(gs_viewer* v, const gs_camera* cam, gs_stream stream) {
  u32 slot = 0;
  const gs_status r = gs_viewer_submit(v, cam, stream, &slot);
  if (r != GS_SUCCESS || v->nslots == 1) return r;
  return gs_viewer_wait(v, slot, stream);
}

gs_status gs_viewer_check(gs_viewer* v, gs_stream stream) {
  if (!v) return GS_ERROR_INVALID_ARGUMENT;
  gs_status worst = GS_SUCCESS;
  for (u32 i = 0; i < v->nslots; ++i) {
    if (gs_viewer_wait(v, i, stream) != GS_SUCCESS) return GS_ERROR_CUDA;
    const gs_status r = gs_context_check(v->slot[i].ctx, stream, nullptr);
    if (r != GS_SUCCESS && worst == GS_SUCCESS) worst = r;
  }
  return worst;
}

gs_status gs_context_set_batch_lanes(gs_context* c, uint32_t lanes) {
  if (!c || lanes > GS_MAX_LANES) return GS_ERROR_INVALID_ARGUMENT;
  if (lanes == c->nlanes) return GS_SUCCESS;
  destroy_lanes(c);
  if (lanes == 0) return GS_SUCCESS;
  if (cudaEventCreateWithFlags(&c->batch_fork, cudaEventDisableTiming) != cudaSuccess) return GS_ERROR_CUDA;
  for (cudaEvent_t& e : c->chunk_done)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      destroy_lanes(c);
      return GS_ERROR_CUDA;
    }
  gs_context_options o{c->max_splats, c->max_width, c->max_height, c->pair_capacity};
  for (u32 l = 0; l < lanes; ++l) {
    gs_status st = gs_context_create(&c->lane[l], &o);
    if (st == GS_SUCCESS && (cudaStreamCreateWithFlags(&c->lane_stream[l], cudaStreamNonBlocking) != cudaSuccess ||
                             cudaEventCreateWithFlags(&c->lane_join[l], cudaEventDisableTiming) != cudaSuccess))
      st = GS_ERROR_CUDA;
    c->nlanes = l + 1;  // what exists so far is torn down on failure
    if (st != GS_SUCCESS) {
      destroy_lanes(c);
      return st;
    }
    gs_context_set_slabs(c->lane[l], c->slab_count, c->slab_end);
    gs_context_set_count_fragments(c->lane[l], c->count_fragments);
    gs_context_set_transmittance_floor(c->lane[l], c->t_floor);
    gs_context_set_train_slab_min(c->lane[l], c->train_slab_min);
    c->lane[l]->lean = true;  // lanes run their views concurrently
  }
  return GS_SUCCESS;
}

gs_status gs_context_set_batch_shared_cull(gs_context* c, int enable) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  c->multi_view_cull = enable != 0;
  return GS_SUCCESS;
}

gs_status gs_render_batched(gs_context* c, const gs_splats* s, uint32_t n_views, const gs_camera* cams,
                            const gs_target* targets, gs_stream stream) {
  if (!c || !s || (n_views && (!cams || !targets))) return GS_ERROR_INVALID_ARGUMENT;
  for (u32 v = 0; v < n_views; ++v) {  // validate everything before enqueueing anything
    if (!targets[v].color_rgba32f && !targets[v].color_bgra8) return GS_ERROR_INVALID_ARGUMENT;
    if (cams[v].width == 0 || cams[v].height == 0) return GS_ERROR_INVALID_ARGUMENT;
    if (cams[v].width > c->max_width || cams[v].height > c->max_height) return GS_ERROR_CAPACITY;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (c->nlanes == 0) {  // one after another on the caller's stream
    for (u32 v = 0; v < n_views; ++v) {
      const gs_status r = gs_render(c, s, &cams[v], &targets[v], nullptr, stream);
      if (r != GS_SUCCESS) return r;
    }
    return GS_SUCCESS;
  }
  if (s->count && (!s->position || !s->cov3d || !s->opacity || !s->sh)) return GS_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(s->sh) & 15u) != 0) return GS_ERROR_INVALID_ARGUMENT;
  if (s->count > c->max_splats || s->count > 0x3fffffffu) return GS_ERROR_CAPACITY;
  if (s->count > 0 && c->multi_view_cull && batch_buffers(c, std::min(n_views, kMaxBatchViews), st)) {
    for (u32 v0 = 0; v0 < n_views; v0 += c->batch_views) {  // groups share the per-view buffers
      const gs_status r = batched_group(c, s, v0, std::min(c->batch_views, n_views - v0), cams, targets, st);
      if (r != GS_SUCCESS) return r;
    }
    c->last_batched = true;
    return GS_SUCCESS;
  }
  const u32 used = std::min(c->nlanes, std::max(n_views, 1u));
  if (cudaEventRecord(c->batch_fork, st) != cudaSuccess) return GS_ERROR_CUDA;
  for (u32 l = 0; l < used; ++l)
    if (cudaStreamWaitEvent(c->lane_stream[l], c->batch_fork, 0) != cudaSuccess) return GS_ERROR_CUDA;
  // Largest views first, each to the lane with the least work so far (work ~ pixels + a fixed cost per
  // view), so the lanes finish together.
  std::vector<u32> order(n_views);
  for (u32 v = 0; v < n_views; ++v) order[v] = v;
  const auto work = [&](u32 v) { return (double)cams[v].width * cams[v].height + 250000.0; };
  std::stable_sort(order.begin(), order.end(), [&](u32 x, u32 y) { return work(x) > work(y); });
  double load[GS_MAX_LANES] = {};
  for (u32 v : order) {
    u32 l = 0;
    for (u32 k = 1; k < used; ++k)
      if (load[k] < load[l]) l = k;
    load[l] += work(v);
    const gs_status r = gs_render(c->lane[l], s, &cams[v], &targets[v], nullptr,
                                  reinterpret_cast<gs_stream>(c->lane_stream[l]));
    if (r != GS_SUCCESS) return r;
  }
  for (u32 l = 0; l < used; ++l) {
    if (cudaEventRecord(c->lane_join[l], c->lane_stream[l]) != cudaSuccess) return GS_ERROR_CUDA;
    if (cudaStreamWaitEvent(st, c->lane_join[l], 0) != cudaSuccess) return GS_ERROR_CUDA;
  }
  c->last_batched = true;
  return GS_SUCCESS;
}

gs_status gs_selftest_bounded_wait(gs_stream stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  void* buf = nullptr;  // 2 status words + the error word
  if (cudaMalloc(&buf, 3 * sizeof(u64)) != cudaSuccess) return GS_ERROR_OUT_OF_MEMORY;
  u32 e = 0;
  const bool ok = cudaMemsetAsync(buf, 0, 3 * sizeof(u64), st) == cudaSuccess &&
                  launch_wait_selftest(static_cast<u64*>(buf), reinterpret_cast<u32*>(static_cast<u64*>(buf) + 2),
                                       st) == cudaSuccess &&
                  cudaMemcpyAsync(&e, static_cast<u64*>(buf) + 2, sizeof(u32), cudaMemcpyDeviceToHost, st) ==
                      cudaSuccess &&
                  cudaStreamSynchronize(st) == cudaSuccess;
  cudaFree(buf);
  if (!ok) return GS_ERROR_CUDA;
  return (e & ERR_TIMEOUT) ? GS_ERROR_DEVICE_TIMEOUT : GS_SUCCESS;
}

gs_status gs_context_check(gs_context* c, gs_stream stream, gs_frame_stats* stats) {
  if (!c) return GS_ERROR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return GS_ERROR_CUDA;
  u32 words[FW_WORDS];
  u32 e = 0;
  if (cudaMemcpy(words, c->frame, sizeof(words), cudaMemcpyDeviceToHost) != cudaSuccess) return GS_ERROR_CUDA;
  if (cudaMemcpy(&e, c->err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return GS_ERROR_CUDA;
  if (cudaMemset(c->err, 0, 4) != cudaSuccess) return GS_ERROR_CUDA;
  if (stats) {
    stats->visible_count = words[FW_VISIBLE];
    stats->tile_pairs = words[FW_PAIR_TOTAL];
    uint64_t ps;
    std::memcpy(&ps, words + FW_PAIR_SUM, 8);
    stats->pairs_emitted = ps;
    uint64_t f[2];
    std::memcpy(f, words + FW_FRAGMENTS, 16);
    stats->fragments = f[0];
    stats->fragments_blended = f[1];
  }
  u32 peak = 0;  // largest slab pair count since the last check (any frame, for capacity growth)
  if (cudaMemcpy(&peak, c->err + 1, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return GS_ERROR_CUDA;
  if (cudaMemset(c->err + 1, 0, 4) != cudaSuccess) return GS_ERROR_CUDA;
  if (stats) stats->tile_pairs = std::max(stats->tile_pairs, peak);
  for (u32 l = 0; l < c->nlanes; ++l) {  // batched frames: errors of every lane, stats summed (pairs: max)
    gs_frame_stats ls{};
    const gs_status r = gs_context_check(c->lane[l], stream, &ls);
    if (r == GS_ERROR_DEVICE_TIMEOUT) e |= ERR_TIMEOUT;
    else if (r == GS_ERROR_INTERNAL) e |= ERR_INTERNAL;
    else if (r == GS_ERROR_CAPACITY) e |= ERR_CAPACITY;
    else if (r != GS_SUCCESS) return r;
    if (stats && c->last_batched) {
      if (l == 0) *stats = gs_frame_stats{};
      stats->visible_count += ls.visible_count;
      stats->tile_pairs = std::max(stats->tile_pairs, ls.tile_pairs);
      stats->fragments += ls.fragments;
      stats->fragments_blended += ls.fragments_blended;
      stats->pairs_emitted += ls.pairs_emitted;
    }
  }
  if (e & ERR_TIMEOUT) return GS_ERROR_DEVICE_TIMEOUT;
  if (e & ERR_INTERNAL) return GS_ERROR_INTERNAL;
  if (e & ERR_CAPACITY) return GS_ERROR_CAPACITY;
  return GS_SUCCESS;
}

// ------------------------------------------------------------------ loader

gs_status gs_parse_ply(const float* rows, uint32_t count, const uint32_t offsets[60], const gs_splat_buffers* out,
                       gs_stream stream) {
  if (!offsets || !out) return GS_ERROR_INVALID_ARGUMENT;
  if (count && (!rows || !out->position || !out->cov3d || !out->opacity || !out->sh)) return GS_ERROR_INVALID_ARGUMENT;
  if (offsets[59] == 0) return GS_ERROR_INVALID_ARGUMENT;
  for (int i = 0; i < 59; ++i)
    if (offsets[i] >= offsets[59]) return GS_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(out->sh) & 3u) != 0) return GS_ERROR_INVALID_ARGUMENT;
  PlyOffsets off;
  std::memcpy(off.v, offsets, sizeof(off.v));
  return from_cuda(launch_parse_ply(rows, count, off, out->position, out->cov3d, out->opacity, out->sh,
                                    reinterpret_cast<cudaStream_t>(stream)));
}

gs_status gs_ply_offsets_from_header(const char* text, size_t length, uint32_t offsets[60], uint64_t* point_count,
                                     size_t* header_bytes) {
  if (!text || !offsets || !point_count || !header_bytes) return GS_ERROR_INVALID_ARGUMENT;
  struct Prop {
    std::string name;
    uint32_t offset;
  };
  Prop props[256];
  int nprops = 0;
  uint32_t offset = 0;
  uint64_t count = 0;
  bool in_vertex = false, saw_end = false, binary_le = false, magic = false;
  size_t pos = 0;
  int line_no = 0;
  while (pos < length) {
    size_t eol = pos;
    while (eol < length && text[eol] != '\n') ++eol;
    std::string line(text + pos, eol - pos);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    pos = eol < length ? eol + 1 : eol;
    if (line_no++ == 0) {
      magic = line == "ply";
      if (!magic) return GS_ERROR_INVALID_ARGUMENT;
      continue;
    }
    if (line == "end_header") {
      saw_end = true;
      break;
    }
    char w0[64] = {0}, w1[64] = {0}, w2[128] = {0};
    const int nw = std::sscanf(line.c_str(), "%63s %63s %127s", w0, w1, w2);
    if (nw < 1) continue;
    if (!std::strcmp(w0, "format")) {
      binary_le = nw >= 2 && !std::strcmp(w1, "binary_little_endian");
    } else if (!std::strcmp(w0, "element")) {
      in_vertex = nw >= 3 && !std::strcmp(w1, "vertex");
      if (in_vertex) count = std::strtoull(w2, nullptr, 10);
    } else if (!std::strcmp(w0, "property") && in_vertex) {
      if (nw < 3 || std::strcmp(w1, "float") != 0 || nprops >= 256) return GS_ERROR_INVALID_ARGUMENT;
      props[nprops].name = w2;
      props[nprops].offset = offset;
      ++nprops;
      offset += 1;
    }
  }
  if (!saw_end || !binary_le || nprops == 0) return GS_ERROR_INVALID_ARGUMENT;
  auto find = [&](const std::string& name, uint32_t* dst) {
    for (int i = 0; i < nprops; ++i)
      if (props[i].name == name) {
        *dst = props[i].offset;
        return true;
      }
    return false;
  };
  bool ok = find("x", &offsets[0]) && find("y", &offsets[1]) && find("z", &offsets[2]) &&
            find("scale_0", &offsets[3]) && find("scale_1", &offsets[4]) && find("scale_2", &offsets[5]) &&
            find("rot_1", &offsets[6]) && find("rot_2", &offsets[7]) && find("rot_3", &offsets[8]) &&
            find("rot_0", &offsets[9]) && find("f_dc_0", &offsets[10]) && find("f_dc_1", &offsets[26]) &&
            find("f_dc_2", &offsets[42]) && find("opacity", &offsets[58]);
  for (int i = 0; ok && i < 15; ++i) {
    ok = find("f_rest_" + std::to_string(i), &offsets[11 + i]) &&
         find("f_rest_" + std::to_string(15 + i), &offsets[27 + i]) &&
         find("f_rest_" + std::to_string(30 + i), &offsets[43 + i]);
  }
  if (!ok) return GS_ERROR_INVALID_ARGUMENT;
  offsets[59] = offset;
  *point_count = count;
  *header_bytes = pos;
  return GS_SUCCESS;
}

// ------------------------------------------------------------------ camera

void gs_camera_perspective(float fovy, float aspect, float znear, float zfar, float out[16]) {
  float p[16] = {0};
  const float t = std::tan(fovy / 2.0f);
  p[0] = 1.0f / (aspect * t);
  p[5] = 1.0f / t;
  p[10] = -(zfar + znear) / (zfar - znear);
  p[11] = -1.0f;
  p[14] = -(2.0f * zfar * znear) / (zfar - znear);
  float conv[16] = {0};
  conv[0] = 1.0f;
  conv[5] = -1.0f;
  conv[10] = 0.5f;
  conv[14] = 0.5f;
  conv[15] = 1.0f;
  gs::mat4_mul_host(conv, p, out);
}

static float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static void normalize3(const float* v, float* o) {
  const float inv = 1.0f / std::sqrt(dot3(v, v));
  o[0] = v[0] * inv;
  o[1] = v[1] * inv;
  o[2] = v[2] * inv;
}

static void cross3(const float* a, const float* b, float* o) {
  o[0] = a[1] * b[2] - b[1] * a[2];
  o[1] = a[2] * b[0] - b[2] * a[0];
  o[2] = a[0] * b[1] - b[0] * a[1];
}

void gs_camera_look_at(const float eye[3], const float center[3], const float up[3], float out[16]) {
  const float d[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
  float f[3], s[3], sn[3], u[3];
  normalize3(d, f);
  cross3(f, up, s);
  normalize3(s, sn);
  cross3(sn, f, u);
  for (int i = 0; i < 16; ++i) out[i] = 0.0f;
  for (int k = 0; k < 3; ++k) {
    out[k * 4 + 0] = sn[k];
    out[k * 4 + 1] = u[k];
    out[k * 4 + 2] = -f[k];
  }
  out[12] = -dot3(sn, eye);
  out[13] = -dot3(u, eye);
  out[14] = dot3(f, eye);
  out[15] = 1.0f;
}

void gs_camera_orbit_eye(const float center[3], float r, float phi, float theta, float out[3]) {
  const float sp = std::sin(phi), cp = std::cos(phi), st = std::sin(theta), ct = std::cos(theta);
  const float d[3] = {sp * st, cp, sp * ct};
  for (int i = 0; i < 3; ++i) out[i] = center[i] + r * d[i];
}

}  // extern "C"
