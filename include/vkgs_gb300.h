/*
 * vkgs_gb300.h -- C ABI of the GB300 (sm_103a) splat pipeline.
 *
 * A drop-in for the per-frame compute-and-indirect-draw path of the vkgs
 * viewer: rank (cull + depth key) -> radix sort -> projection (+SH) -> quad
 * raster + SRC_ALPHA/ONE_MINUS_SRC_ALPHA blend, reimplemented as CUDA kernels.
 * Plain pointers and sizes only; every device pointer is a CUDA device address.
 * All calls that take a stream are asynchronous and stream-ordered; they never
 * synchronise the host.  Device-side failures (a bounded wait that gave up, a
 * capacity overflow) are recorded on the device and returned by
 * gs_context_check().
 *
 * Reference interfaces replaced (paths within jaesung-cs/vkgs):
 *   gs_sorter_*                    vrdxCreateSorter / vrdxGetSorterKeyValueStorageRequirements /
 *                                  vrdxCmdSortKeyValueIndirect / vrdxDestroySorter
 *                                  (src/vkgs/engine/engine.cc:509-521, 1218-1219, 531)
 *   gs_render                      the frame sequence of Engine::Impl::Draw: rank dispatch, sort,
 *                                  inverse map, projection dispatch, indexed-indirect splat draw
 *                                  (src/vkgs/engine/engine.cc:1164-1290, 1380-1498)
 *   gs_parse_ply                   the parse_ply.comp dispatch (engine.cc:1125-1162,
 *                                  src/shader/parse_ply.comp:34-97)
 *   gs_ply_offsets_from_header     the header walk + offset table of SplatLoadThread
 *                                  (src/vkgs/engine/splat_load_thread.cc:53-135)
 *   gs_camera_*                    vkgs::Camera::ProjectionMatrix / ViewMatrix / Eye
 *                                  (src/vkgs/scene/camera.cc:25-45)
 */
#ifndef VKGS_GB300_H
#define VKGS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* gs_stream;

typedef enum gs_status {
  GS_SUCCESS = 0,
  GS_ERROR_INVALID_ARGUMENT = 1, /* null pointer, zero size where one is required, bad layout */
  GS_ERROR_CAPACITY = 2,         /* a size beyond what the context/storage was reserved for */
  GS_ERROR_CUDA = 3,             /* a CUDA runtime call or kernel launch failed */
  GS_ERROR_DEVICE_TIMEOUT = 4,   /* a bounded device-side wait gave up (results of that call are invalid) */
  GS_ERROR_OUT_OF_MEMORY = 5,    /* device allocation failed while reserving */
  GS_ERROR_INTERNAL = 6,         /* a device-side self-check failed (results of that call are invalid) */
} gs_status;

/* Short text for a status code (static storage). */
const char* gs_status_string(gs_status status);

/* ------------------------------------------------------------------------ */
/* Sorter: ascending 32-bit key sort carrying 32-bit values, count on device */
/* ------------------------------------------------------------------------ */

typedef struct gs_sorter gs_sorter;

/* vrdxCreateSorter (engine.cc:509-514).  Binds to the current CUDA device. */
gs_status gs_sorter_create(gs_sorter** sorter);

/* vrdxDestroySorter (engine.cc:531). */
void gs_sorter_destroy(gs_sorter* sorter);

/* vrdxGetSorterKeyValueStorageRequirements (engine.cc:517-519): scratch bytes for sorting up to
 * max_count pairs. */
gs_status gs_sorter_key_value_storage_requirements(gs_sorter* sorter, uint32_t max_count, size_t* bytes);

/* vrdxCmdSortKeyValueIndirect (engine.cc:1218-1219): sorts keys[0..*count) ascending in place and
 * permutes values alongside; equal keys keep their input order (stable).  count lives in device
 * memory and is read on the device (no host sync); *count > max_count is clamped to max_count and
 * recorded as GS_ERROR_CAPACITY on the device.  storage must hold the bytes reported for max_count
 * and must not be used by another sort in flight. */
gs_status gs_sorter_sort_key_value_indirect(gs_sorter* sorter, gs_stream stream, uint32_t max_count,
                                            const uint32_t* count, uint32_t* keys, uint32_t* values,
                                            void* storage, size_t storage_bytes);

/* Reads back and clears the sorter's device error word (synchronises the stream). */
gs_status gs_sorter_check(gs_sorter* sorter, gs_stream stream);

/* No counterpart in the reference.  The same sort for callers that may not allocate device memory
 * (an engine callback that owns the whole memory budget, or code running while other streams are in
 * flight -- cudaMalloc/cudaFree can synchronise the device): no sorter handle, no storage argument,
 * and no cudaMalloc/cudaFree on any path.  Its
 * scratch is one fixed device array inside this library (about 8.4 MB, held by every GPU that
 * loads the library until the process exits), so max_count may not exceed
 * GS_SORT_NOALLOC_MAX_COUNT (GS_ERROR_CAPACITY otherwise).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  The address is kept per device ordinal, i.e. for the device's primary
 * context (the runtime API's context): callers that make another driver-API context current on the
 * same device are not supported.  All calls share the array: calls that may overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller.  device_error (optional device
 * word) receives the error bits: 1 = *count exceeded max_count and was clamped, 2 = a bounded device
 * wait gave up; with device_error NULL those bits are discarded and nothing reports them. */
#define GS_SORT_NOALLOC_MAX_COUNT (1u << 20)
gs_status gs_sort_key_value_noalloc(gs_stream stream, uint32_t max_count, const uint32_t* count, uint32_t* keys,
                                    uint32_t* values, uint32_t* device_error);

/* ------------------------------------------------------------------------ */
/* Splat buffers, camera, target                                             */
/* ------------------------------------------------------------------------ */

/* The reference's SoA splat storage (engine.cc:1639-1651), device pointers. */
typedef struct gs_splats {
  const float* position; /* N x 3 */
  const float* cov3d;    /* N x 6: (00, 10, 20, 11, 21, 22) of the 3D covariance */
  const float* opacity;  /* N, already sigmoid-activated */
  const uint16_t* sh;    /* N x 48 IEEE binary16, [channel][16 coefficients] */
  uint32_t count;
} gs_splats;

/* Writable form of the same buffers, filled by gs_parse_ply. */
typedef struct gs_splat_buffers {
  float* position;
  float* cov3d;
  float* opacity;
  uint16_t* sh;
} gs_splat_buffers;

/* The Camera uniform (src/vkgs/vulkan/shader/uniforms.h:10-15) plus the model push constant
 * (src/shader/rank.comp:13).  Matrices are column-major, like glm::mat4. */
typedef struct gs_camera {
  float projection[16];
  float view[16];
  float camera_position[3];
  uint32_t width;  /* screen_size.x */
  uint32_t height; /* screen_size.y */
  float model[16];
} gs_camera;

/* Colour (+ optional depth) attachment.  At least one colour pointer must be set.
 * The colour attachment is cleared to (0,0,0,1) and splats blend over it in sorted order. */
typedef struct gs_target {
  float* color_rgba32f;    /* H x W x 4 floats, row 0 = top (Vulkan framebuffer origin), or NULL */
  uint8_t* color_bgra8;    /* H x W x 4 bytes B,G,R,A (B8G8R8A8_UNORM of the swapchain), or NULL */
  const float* depth;      /* H x W D32 depth tested with LESS and not written, or NULL = cleared 1.0 */
} gs_target;

/* Optional per-frame outputs, all device pointers (NULL = not requested). */
typedef struct gs_frame_outputs {
  uint32_t* visible_count; /* 1 word: V */
  uint32_t* keys;          /* N words; [0, V) = sorted depth keys floatBitsToUint(1 - ndc.z) */
  uint32_t* index;         /* N words; [0, V) = splat ids in sorted order */
  float* instances;        /* N x 12 floats; [0, V) = projection.comp instance records in sorted order */
  uint32_t* draw_indirect; /* 12 words: the indirect draw arguments of projection.comp:64-75 */
} gs_frame_outputs;

/* ------------------------------------------------------------------------ */
/* Render context                                                            */
/* ------------------------------------------------------------------------ */

typedef struct gs_context gs_context;

typedef struct gs_context_options {
  uint32_t max_splats;      /* N capacity (the reference preallocates MAX_SPLAT_COUNT = 2^23) */
  uint32_t max_width;       /* largest target width */
  uint32_t max_height;      /* largest target height */
  uint32_t max_tile_pairs;  /* (splat, tile) pair capacity; 0 = 16 * max_splats */
} gs_context_options;

typedef struct gs_frame_stats {
  uint32_t visible_count;     /* V of the last frame */
  uint32_t tile_pairs;        /* the max_tile_pairs capacity the last frame needed: its largest depth
                                 slab's (splat, tile) pairs (the differentiable path with stacked slabs:
                                 all slabs' pairs together) */
  uint64_t fragments;         /* covered (pixel, splat) pairs passing the depth test: the fragment-shader
                                 invocations of the reference's draw; only with
                                 gs_context_set_count_fragments(1) */
  uint64_t fragments_blended; /* of those, the ones met front to back while the pixel's transmittance
                                 was still >= the transmittance floor (the blend work actually needed) */
  uint64_t pairs_emitted;     /* (splat, tile) pairs binned and sorted over all slabs of the last frame */
} gs_frame_stats;

/* Creates a context on the current CUDA device and reserves all scratch for the given capacities. */
gs_status gs_context_create(gs_context** context, const gs_context_options* options);

/* The device bytes gs_context_create allocates for these options (the reference preallocates its
 * storage the same way, engine.cc:483-521), computed on the host without a device.  Render lanes,
 * frames in flight and the batched form's per-view buffers allocate on top of it. */
gs_status gs_context_scratch_bytes(const gs_context_options* options, size_t* bytes);
void gs_context_destroy(gs_context* context);

/* Grows the reserved scratch (never shrinks).  Synchronises the device; not for use inside capture. */
gs_status gs_context_reserve(gs_context* context, const gs_context_options* options);

/* No counterpart in the reference (which blends every fragment).  A pixel stops blending once its
 * transmittance T falls below t_floor: everything behind it can then move no channel by more than T,
 * so the image differs from the full blend by less than t_floor per channel.  Default 1e-4 (the
 * threshold of the original 3DGS rasteriser; 39x inside a 1/255 tolerance); valid range
 * (0, 1/255].  The differentiable path stops at the same floor, exactly per pixel. */
gs_status gs_context_set_transmittance_floor(gs_context* context, float t_floor);

/* Makes every following gs_render also count fragments (slower; for statistics and tests). */
gs_status gs_context_set_count_fragments(gs_context* context, int enable);

/* No counterpart in the reference (a scheduling knob of this implementation).  gs_render bins,
 * sorts and blends the depth-sorted splats in up to GS_MAX_SLABS slabs, nearest first, carrying
 * every pixel's blend state from one slab to the next; a 16x16 tile whose pixels all fall below
 * the transmittance floor is finished and receives no pairs from the slabs behind.  ends[i] is the
 * cumulative share of the visible splats in slabs 0..i, in 1/1024 units, strictly increasing,
 * with ends[count-1] = 1024; {1024} is a single slab; the default is {192, 1024}.  The image is the
 * same for every schedule up to the early stop. */
#define GS_MAX_SLABS 4
gs_status gs_context_set_slabs(gs_context* context, uint32_t count, const uint32_t* ends);

/* One frame.  No allocation, no host synchronisation: safe to capture in a CUDA graph once the
 * context holds enough capacity. */
gs_status gs_render(gs_context* context, const gs_splats* splats, const gs_camera* camera,
                    const gs_target* target, const gs_frame_outputs* outputs, gs_stream stream);

/* No counterpart in the reference (its viewer renders one camera per frame).  Renders n_views cameras
 * of the same splats, view v into targets[v] (sizes may differ; each within the context's maxima), as
 * gs_render would one by one.  With render lanes (gs_context_set_batch_lanes), one cull + projection
 * pass over the splats serves 8 views at a time (each splat's data is read once for all of them;
 * per-view outputs identical to gs_render's), largest views first, and each view's depth sort, binning
 * and raster run on a lane as soon as its pass is done (the later passes overlap the lanes' work): sub-contexts with their own scratch and stream, forked from `stream` and joined back
 * into it with events, so the batch is ordered on `stream` and can be captured in a CUDA graph as a
 * whole.  The shared pass keeps every view's records (72 bytes per splat and view, at most 64 views
 * at a time) in an arena allocated by the first batched call that needs it.  A later call that needs
 * a larger arena (more views, or more splats after gs_context_reserve) replaces it, which synchronises
 * the device and frees the old one -- but never while the call is being captured and never once any
 * batched call has been captured with the arena (a captured graph keeps using its addresses): those
 * calls use a per-lane cull instead, with the same results.  With no lanes the views render one after another on
 * `stream`.  gs_context_check afterwards reports every lane's errors and the summed statistics
 * (tile_pairs: the largest). */
gs_status gs_render_batched(gs_context* context, const gs_splats* splats, uint32_t n_views,
                            const gs_camera* cameras, const gs_target* targets, gs_stream stream);

/* No counterpart in the reference.  1 = the plain path's cull + projection streams each 256-splat
 * partition of the splat buffers into shared memory with bulk copies (two partitions in flight per
 * CTA, a control warp resolving the compaction offsets off the compute warps' path); 0 (default) =
 * per-thread loads.  Results are identical.  Staged, the pass alone is faster (0.237 vs 0.254 ms on
 * 6M splats, 66 vs 62 % of HBM bandwidth) and so is a single frame, but its 70 KB of shared memory
 * per CTA keeps other frames' kernels off the SMs while it runs, which costs throughput with frames
 * in flight (4 slots: 763 vs 782 frames/s).  Needs 16-byte aligned position, cov3d, opacity and SH
 * buffers (otherwise the per-thread form runs); not used by the differentiable path (FP32 SH). */
gs_status gs_context_set_cull_staging(gs_context* context, int enable);

/* No counterpart in the reference.  1 = this context's frames run beside other work on the GPU (several
 * contexts rendering on several streams at once): its kernels take launch shapes that leave SM slots to
 * the others -- fewer CTAs per SM for the persistent cull, the onesweep passes and the pair emission,
 * smaller count CTAs, and the raster with two pixels per thread (8x8-pixel warp blocks, the Gaussian and
 * the blend as packed FP32 pairs), which issues fewer instructions per pixel but is slower alone.
 * 0 (default) = shapes for a frame that has the GPU to itself.  Results are identical.  Viewer slots
 * with more than one frame in flight and render lanes always run lean. */
gs_status gs_context_set_lean(gs_context* context, int enable);

/* Batched form: 1 (default) = the shared cull + projection pass above, 0 = each lane culls its views. */
gs_status gs_context_set_batch_shared_cull(gs_context* context, int enable);

/* Creates `lanes` render lanes (0 ... GS_MAX_LANES) with this context's capacities, slab schedule and
 * counting mode (later gs_context_reserve / set_slabs / set_count_fragments calls apply to them too).
 * Synchronises the device and allocates: not for use inside a capture. */
#define GS_MAX_LANES 32
gs_status gs_context_set_batch_lanes(gs_context* context, uint32_t lanes);

/* ------------------------------------------------------------------------ */
/* Differentiable path (no counterpart in the reference viewer)              */
/* ------------------------------------------------------------------------ */

/* Raw per-splat parameters, before activation (device pointers): what a trainer optimises.  The
 * activation is parse_ply.comp's (s = exp(log_scale), q = quat / |quat|, cov3d = R diag(s^2) R^T,
 * opacity = sigmoid(logit)); SH stay FP32. */
typedef struct gs_train_params {
  const float* means;          /* N x 3 */
  const float* log_scales;     /* N x 3 */
  const float* quats;          /* N x 4, (x, y, z, w), any nonzero length */
  const float* opacity_logits; /* N */
  const float* sh;             /* N x 48 FP32, [channel][16 coefficients] */
  uint32_t count;
} gs_train_params;

/* Gradient buffers with the shapes of gs_train_params; gs_train_backward adds into them. */
typedef struct gs_train_grads {
  float* means;
  float* log_scales;
  float* quats;
  float* opacity_logits;
  float* sh;
} gs_train_grads;

/* The frame of gs_render (no caller depth) from raw parameters into an RGBA float
 * target, keeping in the context what gs_train_backward needs: the activated splats, the tile lists,
 * and per pixel its final transmittance and how many list entries it blended (each pixel stops
 * exactly when its transmittance falls below the context's transmittance floor, so the image and the
 * gradients leave out contributions smaller than the floor).  From a splat count on (default 2^20,
 * gs_context_set_train_slab_min) it uses the context's depth-slab schedule and keeps every slab's tile
 * lists (the pair capacity must then hold all slabs' pairs together; gs_frame_stats.tile_pairs reports
 * that need); below it, one slab.  Valid until the context renders again. */
/* Smallest splat count at which the differentiable forward uses depth slabs (default 2^20: below it
 * the per-slab fixed cost outweighs the pairs the slabs save). */
gs_status gs_context_set_train_slab_min(gs_context* context, uint32_t splats);

gs_status gs_train_forward(gs_context* context, const gs_train_params* params, const gs_camera* camera,
                           float* color_rgba32f, gs_stream stream);

/* Gradients of a loss with respect to the raw parameters, given dL/d(image) (H x W x 4 floats) for the
 * last gs_train_forward of this context with the same params and camera.  The blend backward walks
 * each tile's list in reverse from the stored final transmittance (no per-pixel lists are stored) and
 * accumulates per-splat gradients warp-reduced, then atomically; the projection backward then runs per
 * splat through conic -> 2D covariance -> scale / quaternion, SH -> coefficients, and back to the means
 * (including the SH view direction).  Results are added into `grads`.  Returns GS_ERROR_INVALID_ARGUMENT
 * when the context has rendered anything since that forward, or was re-reserved (the forward's lists
 * are gone). */
gs_status gs_train_backward(gs_context* context, const gs_train_params* params, const gs_camera* camera,
                            const float* grad_rgba32f, const gs_train_grads* grads, gs_stream stream);

/* No counterpart in the reference's API: the per-frame loop of Engine::Run (engine.cc:551-601) as a CUDA
 * graph.  gs_viewer_create captures one gs_render of `splats` into `target` with this context (no frame
 * outputs, the target's resolution fixed) on an internal stream; gs_viewer_frame then rewrites the
 * camera constants of the graph's cull node (the only kernel that reads the camera) and launches the
 * graph on `stream`.  Camera width/height must equal the creation camera's.  The context must not be
 * used for other renders while the viewer exists, and timing must be disabled. */
typedef struct gs_viewer gs_viewer;
gs_status gs_viewer_create(gs_viewer** viewer, gs_context* context, const gs_splats* splats, const gs_camera* camera,
                           const gs_target* target);
gs_status gs_viewer_frame(gs_viewer* viewer, const gs_camera* camera, gs_stream stream);
void gs_viewer_destroy(gs_viewer* viewer);

/* Frames in flight, as the reference's viewer keeps them (two, engine.cc:743): the viewer owns
 * frames_in_flight slots (1 ... GS_MAX_FRAMES_IN_FLIGHT), each a captured frame with its own scratch
 * (slot 0 uses `context`, the others own contexts with its capacities and settings), its own stream and
 * its own target (targets[slot]).  gs_viewer_submit puts the next frame into the next slot in turn:
 * it starts after the work enqueued on `stream` so far (and after that slot's previous frame) and does
 * not hold `stream` back, so consecutive frames overlap on the GPU; *slot receives the slot.
 * gs_viewer_wait makes `stream` wait for that slot's latest frame (e.g. before reading its target);
 * a slot's target must not be written by the next frame of that slot before the caller is done with it,
 * which holds when the caller's reads are enqueued on `stream` before the submit that reuses the slot.
 * gs_viewer_frame = submit + wait.  gs_viewer_check waits for every slot on `stream`, synchronises and
 * returns the first device error of the slots' contexts.  With more than one slot the frames are
 * captured with the binning's lean launch shape (fewer count threads and emission CTAs: slower alone,
 * more frames per second when frames overlap); render lanes use it too. */
#define GS_MAX_FRAMES_IN_FLIGHT 8
gs_status gs_viewer_create_frames(gs_viewer** viewer, gs_context* context, const gs_splats* splats,
                                  const gs_camera* camera, const gs_target* targets, uint32_t frames_in_flight);
gs_status gs_viewer_submit(gs_viewer* viewer, const gs_camera* camera, gs_stream stream, uint32_t* slot);
gs_status gs_viewer_wait(gs_viewer* viewer, uint32_t slot, gs_stream stream);
gs_status gs_viewer_check(gs_viewer* viewer, gs_stream stream);

/* The differentiable path over many views of the same splats (no counterpart in the reference): view v
 * is drawn by render lane v (gs_context_set_batch_lanes; n_views may not exceed the lanes,
 * GS_ERROR_CAPACITY otherwise), which keeps that view's forward state; the activation runs once.  The
 * backward runs every view's blend and projection backward concurrently and adds all views' gradients
 * into the one set of buffers (atomically), as a loss summed over the views requires.  Both calls are
 * ordered on `stream` (fork/join over the lanes' streams).  The backward needs the same n_views as the
 * last batched forward, with nothing rendered on the context or its lanes in between (a batched render
 * would overwrite the views' records and lists): GS_ERROR_INVALID_ARGUMENT otherwise. */
gs_status gs_train_forward_batched(gs_context* context, const gs_train_params* params, uint32_t n_views,
                                   const gs_camera* cameras, float* const* colors_rgba32f, gs_stream stream);
gs_status gs_train_backward_batched(gs_context* context, const gs_train_params* params, uint32_t n_views,
                                    const gs_camera* cameras, const float* const* grads_rgba32f,
                                    const gs_train_grads* grads, gs_stream stream);

/* Per-stage GPU timing, the counterpart of the reference's timestamp queries (engine.cc:471-478,
 * 1033-1045).  While enabled, gs_render records CUDA events on its stream around each stage; the
 * events of the last 256 frames are kept.  Stages, in order: cull + key + projection, depth sort,
 * per-tile pair count + scan, pair emission into tile segments, per-tile sort by draw order,
 * raster + blend; the last four are summed over the frame's depth slabs. */
#define GS_NUM_STAGES 6
gs_status gs_context_enable_timing(gs_context* context, int enable);

/* Synchronises the device, then writes up to max_frames rows of GS_NUM_STAGES milliseconds (oldest
 * first) for the frames rendered since timing was enabled, and clears the record.  *frames receives
 * the number of rows written. */
gs_status gs_context_stage_times(gs_context* context, uint32_t max_frames, float* ms, uint32_t* frames);

/* Test support (no reference counterpart): runs one bounded device-side wait on a status word that
 * nothing publishes, so the wait gives up (after about a second of polling) exactly as a look-back
 * whose predecessor never arrives would; synchronises `stream` and returns GS_ERROR_DEVICE_TIMEOUT
 * when the wait recorded its timeout.  Nothing faults, and the device stays usable afterwards. */
gs_status gs_selftest_bounded_wait(gs_stream stream);

/* Synchronises the stream, then returns (and clears) the device error word of the last frames:
 * GS_ERROR_CAPACITY when the tile pairs overflowed (stats->tile_pairs says how many are needed),
 * GS_ERROR_DEVICE_TIMEOUT when a bounded wait gave up.  stats may be NULL. */
gs_status gs_context_check(gs_context* context, gs_stream stream, gs_frame_stats* stats);

/* ------------------------------------------------------------------------ */
/* Loader: PLY header and parameter activation                               */
/* ------------------------------------------------------------------------ */

/* Walks an ASCII PLY header (up to and including "end_header") and fills the 60-word offset table of
 * splat_load_thread.cc:114-135 (float offsets of x..z, scale_0..2, rot_1,rot_2,rot_3,rot_0, the 48 SH
 * terms in [channel][coefficient] order, opacity, and the row stride at [59]).  Every property must
 * be "float".  *header_bytes receives the size of the header including its final newline. */
gs_status gs_ply_offsets_from_header(const char* text, size_t length, uint32_t offsets[60],
                                     uint64_t* point_count, size_t* header_bytes);

/* parse_ply.comp: activates count PLY rows (device, offsets[59] floats each) into the splat buffers:
 * s = exp(log s), q normalised, cov3d = R S^2 R^T, SH to binary16 (round to nearest even),
 * opacity = sigmoid. */
gs_status gs_parse_ply(const float* rows, uint32_t count, const uint32_t offsets[60],
                       const gs_splat_buffers* out, gs_stream stream);

/* ------------------------------------------------------------------------ */
/* Camera helpers (host only)                                                */
/* ------------------------------------------------------------------------ */

/* glm::perspective(fovy, aspect, near, far) (right-handed, clip z in [-1,1]) followed by the
 * gl-to-vulkan conversion of camera.cc:29-34 (y flipped, z' = z/2 + w/2). */
void gs_camera_perspective(float fovy, float aspect, float znear, float zfar, float out[16]);

/* glm::lookAt(eye, center, up), right-handed. */
void gs_camera_look_at(const float eye[3], const float center[3], const float up[3], float out[16]);

/* Camera::Eye: center + r * (sin phi sin theta, cos phi, sin phi cos theta). */
void gs_camera_orbit_eye(const float center[3], float r, float phi, float theta, float out[3]);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
uint32_t gs_version(void);

#ifdef __cplusplus
}
#endif

#endif /* VKGS_GB300_H */
