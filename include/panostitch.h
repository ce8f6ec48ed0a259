/*
 * panostitch.h -- C ABI of the GB300 panorama stitch path.
 *
 * The path: per camera frame, apply the exposure / white-balance LUTs, warp
 * through precomputed dst->src maps with bilinear sampling into an
 * equirectangular canvas, then blend all cameras with the integer multiband
 * pipeline (Gaussian pyramids of the seam weights, Laplacian pyramids of the
 * warped frames, weighted accumulation, normalisation, collapse) and write
 * 8-bit BGR.
 *
 * Every entry point returns an int status (PS_OK or a PS_E* code) and never
 * throws; ps_last_error() returns the thread-local message of the last
 * failure.  Work is ordered on the caller's CUDA stream (NULL = the legacy
 * default stream): the renders run on their own streams, and the caller's
 * stream waits for each call's completion; no entry point synchronises the
 * stream unless it says so.  A ps_render is not thread-safe; distinct
 * renders may be used from different threads.  A render records its launch
 * sequence as a CUDA graph with stream capture (on its first frames, after
 * prepare or a launch-shape change, and throughout ps_render_autotune);
 * CUDA forbids synchronising the whole device or context while any of its
 * streams captures, so threads that share a device with renders wait on
 * their own streams or events, not with cudaDeviceSynchronize.
 *
 * Each declaration names the reference interface it replaces
 * (xpngzhng/PanoStitcher, path:line).
 */
#ifndef PANOSTITCH_H
#define PANOSTITCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define PS_OK 0
#define PS_EINVAL 1    /* bad argument / precondition (sizes, formats, counts) */
#define PS_ENOMEM 2    /* device or host allocation failed, or budget exceeded */
#define PS_ECUDA 3     /* a CUDA runtime call failed */
#define PS_ETIMEOUT 4  /* a bounded wait ran out */
#define PS_ESTATE 5    /* object not prepared / already running / closed */

#define PS_MAX_LEVELS 16   /* getTrueNumLevels cap, source/Blend/MultiBandBlend.cpp:325 */
#define PS_MAX_CAMS 64     /* cameras per rig */
#define PS_MAX_IN_FLIGHT 8 /* frames of one render in flight (state slots) */

/* PhotoParam, source/Warp/ZReproject.h:17-50 (same fields, same order,
   same meaning: image_type 0 rectilinear, 1 full-frame fisheye,
   2 drum fisheye, 3 circular fisheye; angles in degrees). */
typedef struct ps_photo_param {
    int image_type, crop_mode, crop_x, crop_y, crop_width, crop_height;
    int circle_x, circle_y, circle_r;
    double hfov, vfov, alpha, beta, gamma, shift_x, shift_y, shear_x, shear_y;
    double yaw, pitch, roll;
} ps_photo_param;

/* Pixel formats (B,G,R byte order like cv::Mat CV_8UC3 / CV_8UC4). */
#define PS_FMT_BGR24 24
#define PS_FMT_BGR32 32   /* 4th byte ignored on input, written as 0 */
/* Where an image lives. */
#define PS_MEM_HOST 0     /* host memory; pinned memory gives async copies */
#define PS_MEM_DEVICE 1   /* device memory of the current device */

/* An image view: the POD replacement of cv::Mat / cv::cuda::GpuMat. */
typedef struct ps_image {
    void* data;
    long long pitch;     /* bytes between rows */
    int width, height;
    int format;          /* PS_FMT_* */
    int location;        /* PS_MEM_* */
} ps_image;

/* Planar encoder formats (BT.601 studio range, the encoders' inputs in
   source/Task/PanoramaLocalDiskTask.cpp:2054-2076). */
#define PS_FMT_YUV420P 420  /* planes: Y (w x h), U (w/2 x h/2), V (w/2 x h/2) */
#define PS_FMT_NV12 12      /* planes: Y (w x h), interleaved U,V (w bytes x h/2) */

/* A planar frame view: the replacement of the Y / U / V (or Y / UV)
   GpuMats and the encoder's host planes. */
typedef struct ps_planar_image {
    void* planes[3];        /* Y, U, V (YUV420P) or Y, UV, unused (NV12) */
    long long pitches[3];   /* bytes between rows of each plane */
    int width, height;      /* luma size; both even */
    int format;             /* PS_FMT_YUV420P or PS_FMT_NV12 */
    int location;           /* PS_MEM_* (all planes alike) */
} ps_planar_image;

/* Thread-local text of the last error ("" if none). */
const char* ps_last_error(void);
/* Library version string. */
const char* ps_version(void);

/* ==== the render: CudaPanoramaRender2 (source/Task/RicohUtil.h:193-220) ==== */
typedef struct ps_render ps_render;

/* Construct an empty render (CudaPanoramaRender2::CudaPanoramaRender2). */
int ps_render_create(ps_render** out);
/* Destroy; NULL is a no-op (~CudaPanoramaRender2).  Waits for the render's
   frames in flight first (its own work only, not the whole device). */
void ps_render_destroy(ps_render* r);

/* CudaPanoramaRender2::prepare (source/Task/RicohUtil.cpp:1091-1205) with the
   camera parameters passed directly instead of a file path.  Preconditions
   as the reference: dst_w, dst_h even and dst_h * 2 == dst_w; blend_param
   > 0.  high_quality_blend non-zero prepares the multiband path with
   blend_param the maximum number of levels; 0 prepares the linear-blend
   path (RicohUtil.cpp:1174-1193): blend_param (<= 1024) is the radius of the
   Gaussian that feathers the seam masks into per-camera weights
   (getWeightsLinearBlend32F, source/Blend/LinearBlend.cpp:136-151), and
   render accumulates the weighted warped frames in fp32
   (cudaReprojectWeightedAccumulateTo32F + convertTo, RicohUtil.cpp:1269-1286;
   BGR output only).  Seam masks follow
   the rule set by ps_render_set_seam_rule (by default the nearest optical
   axis).  Synchronises the stream. */
int ps_render_prepare(ps_render* r, const ps_photo_param* params, int num_params, int high_quality_blend,
                      int blend_param, int src_w, int src_h, int dst_w, int dst_h, void* stream);
/* CudaPanoramaRender2::prepare(path, ...) itself: the camera parameters
   are read from a PTGui .pts file as loadPhotoParams does
   (source/Warp/PhotoParam.cpp:681-771).  The reference's XML camera files
   need ticpp and are PS_EINVAL here, as is a file without cameras ("load
   photo params failed", RicohUtil.cpp:1111-1116). */
int ps_render_prepare_file(ps_render* r, const char* path, int high_quality_blend, int blend_param, int src_w,
                           int src_h, int dst_w, int dst_h, void* stream);
/* loadPhotoParams alone: writes up to capacity parameters and the number
   found to *num (0 when the file holds no usable cameras). */
int ps_load_photo_params(const char* path, ps_photo_param* params, int capacity, int* num);

/* Same, with explicit seam (unique) masks: num_params host arrays of
   dst_h*dst_w uint8 (non-zero = owned), each a subset of that camera's
   coverage; they replace getNonIntersectingMasks
   (source/CudaAccel/CudaMultibandBlend.cpp:570-571) and, like its masks,
   must not intersect (PS_EINVAL naming the first shared pixel). */
int ps_render_prepare_with_seams(ps_render* r, const ps_photo_param* params, int num_params,
                                 int high_quality_blend, int blend_param, int src_w, int src_h, int dst_w,
                                 int dst_h, const uint8_t* const* seam_masks, void* stream);

/* CudaPanoramaRender2::render (source/Task/RicohUtil.cpp:1207-1339).
   src: num_src camera frames (BGR24 or BGR32, host or device, all src_w x
   src_h).  luts: NULL (no correction) or num_luts == num_images tables of
   3*256 bytes (B, G, R), host memory; a malformed count is PS_EINVAL (the
   reference logs a warning and skips the correction).  dst: a dst_w x dst_h
   BGR32 or BGR24 image, host or device.  Host src / dst are copied inside
   the call (pinned memory keeps the copies asynchronous); device src / dst
   are read / written in place.  The work runs on the render's own copy-in,
   compute and copy-out streams, and the caller's stream waits for its
   completion.  A render keeps a set of per-frame state per frame in flight
   (ps_render_set_frames_in_flight; eight by default), so that many calls
   can be in flight: with host src and dst a call does not wait for the
   caller's earlier work (consecutive calls overlap their uploads, kernels
   and downloads); with device src or dst it waits for the caller's stream,
   so calls on different streams overlap.  Host src and dst must stay
   untouched until the caller's stream reaches the call.  Does not
   synchronise. */
int ps_render_render(ps_render* r, const ps_image* src, int num_src, const uint8_t* luts, int num_luts,
                     ps_image* dst, void* stream);

/* CudaPanoramaRender2::render followed by the encoder handoff
   cvtBGR32ToYUV420P / cvtBGR32ToNV12 and the planes' download
   (source/CudaAccel/ImageProc.cu:44-160, called at
   source/Task/PanoramaLocalDiskTask.cpp:2054-2076), in one call: the
   conversion is fused into the level-0 blend store, so the BGR canvas is
   never written.  The planes are byte-identical to converting the
   ps_render_render BGR32 output.  dst: dst_w x dst_h, host or device.  Does
   not synchronise. */
int ps_render_render_yuv(ps_render* r, const ps_image* src, int num_src, const uint8_t* luts, int num_luts,
                         const ps_planar_image* dst, void* stream);

/* Seam (unique mask) rule of the next prepare without explicit seams:
   PS_SEAMS_NEAREST_AXIS (default) gives each covered pixel to the camera
   whose optical axis is nearest; PS_SEAMS_DISTANCE is the reference's
   getNonIntersectingMasks (source/Blend/Mask.cpp:376-398, called at
   source/CudaAccel/CudaMultibandBlend.cpp:570-571), which splits overlaps
   by the L1 distance to each coverage border.  Any other value is
   PS_EINVAL. */
#define PS_SEAMS_NEAREST_AXIS 0
#define PS_SEAMS_DISTANCE 1
int ps_render_set_seam_rule(ps_render* r, int rule);
/* Custom masks (CudaTilingMultibandBlendFast::blend(images, masks, blendImage),
   source/CudaAccel/CudaMultibandBlend.cpp:825-893, as the Tasks call it per
   frame with each camera's custom mask of the frame's interval or else its
   unique mask, source/Task/PanoramaPreviewTask.cpp:382-400): the frames
   rendered after this call weight the cameras by num_masks host uint8
   masks (dst_w x dst_h, non-zero = weight 256) instead of the unique masks,
   normalise by the weight sums whatever the coverage, and are zero outside
   the masks' union.  The masks may overlap.  The reference rebuilds the
   weight pyramids on every such frame; here they are rebuilt once per mask
   set, since the masks change only between intervals.  masks = NULL (and
   num_masks 0) returns to the unique masks.  Waits for the render's frames
   in flight; synchronises.  Multiband blend only: a linear-blend render is
   PS_EINVAL (the reference warns and ignores them, RicohUtil.cpp:929-930). */
int ps_render_set_custom_masks(ps_render* r, const uint8_t* const* masks, int num_masks, void* stream);
/* Frames in flight, 1..PS_MAX_IN_FLIGHT (default PS_MAX_IN_FLIGHT): the sets
   of per-frame state (pyramids, staging) the next prepare allocates.  Fewer
   save device memory; more let consecutive renders overlap on the GPU.
   No reference counterpart (the reference renders one frame at a time). */
int ps_render_set_frames_in_flight(ps_render* r, int n);
/* The reference's prepare estimates the device memory of its stream-based
   render and, when the free memory exceeds it by less than 500 MB, renders
   one camera at a time instead (source/Task/RicohUtil.cpp:1135-1170,
   1315-1329).  Here the per-frame state is per frame in flight, so the
   multiband prepare takes as many frames in flight (of those asked for) as
   fit the free memory with that 500 MB margin, down to one, and reports the
   fallback through ps_render_is_low_memory.  ps_render_set_memory_budget
   caps that room further for the next prepare (bytes; 0 = free memory
   only); ps_render_get_frames_in_flight gives the count taken.  Every count
   stitches the same bytes. */
int ps_render_set_memory_budget(ps_render* r, long long bytes);
int ps_render_is_low_memory(const ps_render* r);
/* The map-free remap of the reference's low-memory path
   (cudaReprojectTo16S(src, dst, dstSize, param), source/CudaAccel/
   CudaReproject.cu:559-602,722-742, which computes dstToSrc per pixel).
   With enable != 0 the next multiband prepare keeps no maps: the remap
   computes each pixel's source coordinate in fp32 from the camera
   parameters (the reference's dstToSrc does it in double, which GB300 runs
   at a small fraction of its fp32 rate), and takes the coverage from the
   FP64 geometry of prepare.  Level 0 is then within +-1 of the exact remap
   per channel, not bit for bit, and the blend of it is exact.  prepare also
   turns it on by itself when even one frame in flight with resident maps
   does not fit (ps_render_is_low_memory).  ps_render_is_map_free reports
   the mode of the last prepare.  The maps cannot be exported then. */
int ps_render_set_map_free(ps_render* r, int enable);
int ps_render_is_map_free(const ps_render* r);
/* The prepared render's frames in flight (0 before prepare). */
int ps_render_get_frames_in_flight(const ps_render* r);
/* CudaPanoramaRender2::render with decoder frames: src holds num_src YUV420P
   or NV12 frames (BT.601 studio range, src_w x src_h, host or device, each
   its own format), converted on the device to BGR32 as cvtYUV420PToBGR32 /
   cvtNV12ToBGR32 do (source/CudaAccel/ImageProc.cu:165-259) and then
   stitched as ps_render_render stitches BGR32 frames.  Host frames cross
   the host link at 1.5 bytes per pixel instead of 4.  Exactly one of dst
   (as ps_render_render) and ydst (as ps_render_render_yuv) is given.  The
   first call allocates the render's planar staging (1.5 bytes per source
   pixel per camera and frame in flight).  Streams and lifetimes as
   ps_render_render. */
int ps_render_render_planar(ps_render* r, const ps_planar_image* src, int num_src, const uint8_t* luts,
                            int num_luts, const ps_image* dst, const ps_planar_image* ydst, void* stream);

/* Launch the per-frame kernels as one captured CUDA graph (default 1) or as
   individual launches (0).  No reference counterpart. */
int ps_render_set_graph(ps_render* r, int enabled);

/* The render's seam (unique) masks into num host buffers of dst_w * dst_h
   bytes (0 / 255): what the reference's render keeps as dstUniqueMasksGPU
   and its Tasks take from the blender's getUniqueMasks
   (source/CudaAccel/CudaMultibandBlend.cpp:895-901). */
int ps_render_get_unique_masks(const ps_render* r, uint8_t* const* masks, int num);
/* The device bytes a render of this rig would hold with frames_in_flight
   state slots (1..8), an upper bound that assumes every camera covers the
   whole canvas; no allocation.  The reference's prepare makes the same kind
   of estimate against the free device memory to choose its low-memory path
   (source/Task/RicohUtil.cpp:1135-1170); ps_render_prepare makes it too
   (see ps_render_set_frames_in_flight).  -1 on bad arguments. */
long long ps_render_estimate_memory(const ps_photo_param* params, int num_params, int blend_param, int src_w,
                                    int src_h, int dst_w, int dst_h, int frames_in_flight);

/* Failure status of the render's kernels.  No reference counterpart (the
   reference's kernels have no waits that can run out).  Every wait of the
   blend kernels on the bulk-copy ring is bounded; one that runs out sets a
   status bit on every frame of its launch and the kernel carries on, so the
   device stays usable.  ps_render_check waits for the render's frames in
   flight, reads and clears that status, and returns PS_ETIMEOUT if a wait ran
   out since the last check (those frames may be wrong), else PS_OK. */
int ps_render_check(ps_render* r);
/* Failure-path test hook, no reference counterpart: with polls > 0 every
   blend launch of this render makes one wait of that many polls on a
   barrier that nothing completes, so that wait runs out and
   ps_render_check reports PS_ETIMEOUT.  0 (default) turns it off.  Waits
   for the frames in flight; the next render re-records its launches. */
int ps_render_set_wait_probe(ps_render* r, int polls);

/* CudaPanoramaRender2::clear / getNumImages (source/Task/RicohUtil.cpp:1341-1361).
   clear, like a new prepare, waits for the render's frames in flight before
   it frees their state. */
void ps_render_clear(ps_render* r);
int ps_render_get_num_images(const ps_render* r);

/* Introspection (no reference counterpart; used by tests and admission). */
int ps_render_get_num_levels(const ps_render* r);
int ps_render_is_full_mask(const ps_render* r);
long long ps_render_resident_bytes(const ps_render* r);
/* Device-resident frame buffers owned by the render (BGR32, pitch in
   bytes), one per camera: writing frames there and passing them as device
   src avoids any copy.  They also stage host sources of every other render
   call, so do not mix the two on one render. */
int ps_render_get_input_buffer(ps_render* r, int cam, void** data, long long* pitch);
/* Copies of the prepared state to host memory, for parity checks:
   what: 0 x map (float, dst_h*dst_w, -1 where invalid), 1 y map (float),
   2 coverage mask (uint8 0/255), 3 seam mask (uint8 0/255),
   4 weight pyramid level `level` (int16), 5 alpha pyramid level `level`
   (int32, the raw 5x5 sum as pyrDown16SC1To32SC1 writes it; level >= 1),
   6 linear-blend weight (float, linear-blend mode), 7 level 0 of the last
   render (uint8 x4 B,G,R,0 per pixel: the remap's output; synchronises). */
int ps_render_export(const ps_render* r, int what, int cam, int level, void* host_out, long long bytes);
/* Debug copy of the collapsed result at level `level` >= 1 of the last
   render (int16 x4 per pixel), for bit-exact checks of the pipeline. */
int ps_render_export_collapsed(const ps_render* r, int level, int16_t* host_out, long long bytes, void* stream);

/* Measurement hooks (no reference counterpart).  While profiling is on,
   renders launch step by step with a CUDA event pair around every launch
   (no graph); ps_render_profile_read aggregates the finished launches of
   one kernel kind (0 remap, 1 pyrDown, 2 blend, 3 the tail kernel that runs
   the few-tile top levels, reported at its lowest blend level, 4 the
   linear-blend render, 5 the conversion of decoder frames, at level 0, 6
   the blend of few-tile levels in half tiles, 7 the exact recompute of the
   remap pixels whose fp32 result lies near a rounding tie, at level 0) at
   one level (-1 = all levels): launch count, summed device milliseconds
   and summed algorithmic bytes (each input and output element counted
   once).
   Enabling resets the aggregates. */
int ps_render_profile(ps_render* r, int enable);
int ps_render_profile_read(ps_render* r, int kind, int level, long long* launches, double* total_ms,
                           double* bytes);
/* Kernel launches one render issues. */
int ps_render_launches_per_frame(const ps_render* r);
/* Algorithmic bytes of one frame: camera frames (bytes_in_per_px each), the
   maps of covered canvas pixels (8 B), the non-zero seam weights (2 B) and
   alpha divisors (4 B) of every level, and the canvas (bytes_out_per_px).
   Returns < 0 if the render is not prepared. */
double ps_render_algorithmic_bytes(const ps_render* r, int bytes_in_per_px, int bytes_out_per_px);

/* ==== launch shapes and the autotuner (no reference counterpart: CudaAccel
   fixes its launch shapes at compile time, e.g. the 16x16 blocks of
   source/CudaAccel/CudaPyramid2.cu:989-1016) ==== */
/* The launch choices that can change after prepare.  Tile sizes stay fixed
   (32x16 remap and pyrDown tiles, 64x16 blend tiles); every shape gives the
   same output bytes. */
typedef struct ps_launch_shape {
    int tail_max_items;   /* pyramid levels (from the top) with at most this many
                             tiles run in the one-cluster tail kernel; 0 = no tail
                             (default 16) */
    int tail_cluster;     /* CTAs per rig in the tail kernel: 8, 16, or 0 = the
                             widest the GPU co-schedules (default 0) */
    int tail_half_tiles;  /* 1: the tail blends levels above 0 in 64x8 half tiles,
                             two pixels per thread; 0: whole tiles (default 1) */
    int ctas_per_sm[3];   /* CTAs per SM of the remap, pyrDown and blend kernels'
                             one-wave grids; 0 = as many as fit (default 0) */
    int small_blend_max_items; /* blend levels above 0 (below the tail) with at
                             most this many tiles run as 64x8 half tiles, up to
                             eight cameras staged at once; 0 = none (default 0) */
    int remap_defer_ties; /* 1: the remap lists the pixels whose fp32 result lies
                             near a rounding tie and a short second launch
                             recomputes them exactly (faster with frames in
                             flight); 0: the remap recomputes them itself (the
                             shortest single frame) (default 1) */
} ps_launch_shape;
typedef struct ps_tune_report {
    double ms_per_frame_default;  /* device ms per frame of the default shape */
    double ms_per_frame_chosen;   /* device ms per frame of the chosen shape */
    int trials;                   /* timed runs (0 when the result was cached) */
    int cached;                   /* 1: an earlier tuning of the same geometry */
} ps_tune_report;
/* Set before prepare, the shape applies at prepare; set after, the call waits
   for the render's frames in flight and the next render re-records its launches.
   Out-of-range fields: PS_EINVAL. */
int ps_render_set_launch_shape(ps_render* r, const ps_launch_shape* shape);
int ps_render_get_launch_shape(const ps_render* r, ps_launch_shape* shape);
/* Times launch shapes on the prepared render (frames_per_trial frames per
   timed run, 0 = 20; issued round-robin on in_flight streams, 0 = the
   render's frames in flight) over a small grid of the interacting
   choices, then by coordinate descent from the best, and keeps the fastest.  The render's input staging (every state
   slot) is overwritten with test patterns, and the trials cycle through
   them as distinct frames would.  A geometry tuned before in this
   process is not timed again unless force is non-zero.  Blocks (a few
   seconds at 4096x2048).  chosen and report may be NULL. */
int ps_render_autotune(ps_render* r, int frames_per_trial, int in_flight, int force, ps_launch_shape* chosen,
                       ps_tune_report* report);

/* ==== batched render: several rigs, one frame each, in one launch sequence ==== */
/* All rigs' work goes into shared persistent launches (one per pyramid step)
   captured once per batch composition as a CUDA graph.  Each rig keeps its
   own tail split; a launch's grid and cluster widths are the widest any of
   its rigs' launch shapes asks for.  srcs[k] holds
   ps_render_get_num_images(renders[k]) frames.  No reference counterpart
   (the reference renders one rig per call, source/Task/RicohUtil.cpp:1207). */
int ps_render_batch(ps_render* const* renders, int num_renders, const ps_image* const* srcs,
                    const uint8_t* const* luts, ps_image* dsts, void* stream);

/* ==== CudaAccel primitives (source/CudaAccel/CudaInterface.h) ==== */
/* cudaGenerateReprojectMapAndMask (CudaInterface.h:130-131, kernel
   source/CudaAccel/CudaReproject.cu:81-290): double-precision dst->src
   maps on the GPU, -1 where invalid, and a 0/255 coverage mask.
   Device outputs, tightly packed dst_h*dst_w. */
int ps_generate_reproject_map_and_mask(const ps_photo_param* param, int src_w, int src_h, int dst_w, int dst_h,
                                       float* xmap, float* ymap, uint8_t* mask, void* stream);
/* cudaTransform + cudaReprojectTo16S fused (CudaInterface.h:120-121 and
   :150-151): LUT (3*256 device bytes or NULL) on each source texel, then
   bilinear interpolation through float maps, written as int16 x4 (B,G,R,0;
   0 where the map is invalid).  All pointers device; pitches in bytes. */
int ps_reproject_to_16s(const ps_image* src, const float* xmap, const float* ymap, long long map_pitch,
                        int dst_w, int dst_h, const uint8_t* lut, int16_t* dst, long long dst_pitch,
                        void* stream);
/* getLUT (source/Blend/ExposureColorOptimize.cpp:1217-1223) on the host. */
int ps_get_lut(double k, uint8_t* lut256);
/* getNonIntersectingMasks (source/Blend/Mask.cpp:376-398): num device
   coverage masks (width x height each, non-zero = covered, packed one after
   another) -> num device 0/255 unique masks (same layout): a partition of
   the union of the coverage in which camera i, in index order, takes the
   pixels where its own L1 distance to an uncovered pixel exceeds that of
   the union taken before it.  Allocates scratch; synchronises. */
int ps_non_intersecting_masks(const uint8_t* masks, int num, int width, int height, uint8_t* out, void* stream);
/* cv::distanceTransform(mask, dist, CV_DIST_L1, 3) on the device: the exact
   L1 distance of every pixel to the nearest zero pixel of the mask, as
   int32; a mask without zero pixels gives values >= 2^28.  Device
   pointers, tightly packed. */
int ps_distance_transform_l1(const uint8_t* mask, int width, int height, int32_t* dist, void* stream);
/* cvtBGR32ToYUV420P / cvtBGR32ToNV12 (source/CudaAccel/ImageProc.cu:97-160):
   a device BGR32 image to device planes of the same (even) size.  Y per
   pixel; U and V per 2x2 block from its left column, as the reference
   computes them. */
int ps_cvt_bgr32_to_yuv(const ps_image* src, const ps_planar_image* dst, void* stream);
/* cvtYUV420PToBGR32 / cvtNV12ToBGR32 (source/CudaAccel/CudaInterface.h:
   167-171, kernels source/CudaAccel/ImageProc.cu:165-222): device planes of
   an even-sized frame to a device BGR32 image of the same size, BT.601
   studio range in 20-bit fixed point; the fourth byte is written 0 (the
   reference leaves it unwritten). */
int ps_cvt_yuv_to_bgr32(const ps_planar_image* src, const ps_image* dst, void* stream);

/* No counterpart in the reference.  The nearest-optical-axis seam masks of a
   rig (the masks ps_render_prepare derives internally), computed without
   allocating any device memory, for callers that cannot call cudaMalloc: a
   host whose device memory is owned by another allocator, or a real-time
   thread that must not risk the synchronisation an allocation can cause.
   The caller passes the camera parameters and the output: seams, device
   memory of num_params * dst_h * dst_w bytes (0/255 per camera).  The
   scratch (parameters and coverage masks) lives in one fixed 16 MiB device
   array inside the library, held on every GPU that loads it until the
   process exits; num_params * dst_w * dst_h must not exceed
   16 MiB - 64 KiB, and dst_h must not exceed 65535, else PS_EINVAL.  The
   camera parameters reach the device as a kernel argument, so nothing of
   the caller's host memory is read after the call returns.  The first call
   on a device looks up the array's address on that device, so make it
   before any stream capture.  All calls on a device share the array: calls
   whose work overlaps on the GPU race.  Every scratch byte a call reads it
   has written itself. */
int ps_nearest_axis_seams_no_alloc(const ps_photo_param* params, int num_params, int src_w, int src_h, int dst_w,
                                   int dst_h, uint8_t* seams, void* stream);

/* The bounds-checked build (no reference counterpart): libpanostitch_checked.so
   is the same library with every global access of the stitch kernels checked
   against the extent of its buffer; an access outside is not made and is
   counted.  Returns the count since the last reset (waits for the device),
   or -1 in the normal build.  reset != 0 sets it back to 0. */
long long ps_debug_bounds_violations(int reset);

/* ==== multiband blender: CudaTilingMultibandBlendFast (CudaInterface.h:45-82) ==== */
typedef struct ps_blender ps_blender;
int ps_blender_create(ps_blender** out);
void ps_blender_destroy(ps_blender* b);
/* prepare(masks, maxLevels, minLength) (source/CudaAccel/CudaMultibandBlend.cpp:
   549-642): masks = num host uint8 coverage masks (width x height), seams =
   num host uint8 unique masks (subsets of the masks that do not intersect,
   else PS_EINVAL), or NULL to derive them from the masks with
   getNonIntersectingMasks as the reference does (:570-571).  Synchronises. */
int ps_blender_prepare(ps_blender* b, const uint8_t* const* masks, const uint8_t* const* seams, int num,
                       int width, int height, int max_levels, int min_length, void* stream);
/* blend(images, blendImage) (:785-823): num device images of int16 x4
   (CV_16SC4, values 0..255 in B,G,R as cudaReprojectTo16S writes them) or
   BGR32 uint8 (CV_8UC4) -> dst (device, BGR32 or BGR24).  A 16-bit value
   outside 0..255 is PS_EINVAL (checked on the device; the status is read
   back, so this call synchronises when image_format is 16). */
int ps_blender_blend(ps_blender* b, const void* const* images, const long long* pitches, int image_format,
                     ps_image* dst, void* stream);
int ps_blender_get_num_levels(const ps_blender* b);
/* CudaTilingMultibandBlendFast::begin / tile / end (source/CudaAccel/
   CudaInterface.h:51-53, CudaMultibandBlend.cpp:737-783): the blend fed one
   camera at a time, as the reference's render does when device memory is
   short (source/Task/RicohUtil.cpp:1315-1329).  begin starts a blend; tile
   takes camera `index`'s level-0 image (device int16 x4 or BGR32 uint8, as
   ps_blender_blend; checked the same way, so it synchronises) and is done
   with it when it returns, so one caller buffer can serve every camera; end
   blends into dst (device, BGR32 or BGR24).  begin + a tile of every camera
   + end gives exactly the bytes of ps_blender_blend.  A camera not tiled
   contributes nothing while its weights still count in the normalisation,
   as in the reference.  Stricter than the reference: a camera tiled twice
   since begin, tile or end without begin, and another blend between begin
   and end are errors (PS_EINVAL / PS_ESTATE). */
int ps_blender_begin(ps_blender* b, void* stream);
int ps_blender_tile(ps_blender* b, const void* image, long long pitch, int image_format, int index, void* stream);
int ps_blender_end(ps_blender* b, ps_image* dst, void* stream);
/* getUniqueMasks (CudaMultibandBlend.cpp:895-901): the seam (unique) masks,
   into num host buffers of width * height bytes (0 / 255). */
int ps_blender_get_unique_masks(const ps_blender* b, uint8_t* const* masks, int num);
/* calcUsedMemorySize (:903-920): device bytes the blender holds. */
long long ps_blender_used_memory(const ps_blender* b);
/* estimateMemorySize (:922-926): device bytes a blender of this size would
   hold at most, whatever the masks (no allocation); -1 on bad arguments. */
long long ps_blender_estimate_memory(int width, int height, int num_images, int max_levels);
/* As ps_render_check / ps_render_set_wait_probe, for the blender's blends. */
int ps_blender_check(ps_blender* b);
int ps_blender_set_wait_probe(ps_blender* b, int polls);
/* blend(images, masks, blendImage) (:825-893): later blends use num host
   uint8 custom masks (width x height) as ps_render_set_custom_masks
   describes; masks = NULL returns to the unique masks.  Synchronises. */
int ps_blender_set_custom_masks(ps_blender* b, const uint8_t* const* masks, int num_masks, void* stream);

/* ==== serving loop: live streams with continuous batching ==== */
typedef struct ps_server ps_server;
/* budget_bytes: device memory that resident stream state may occupy
   (admission control, like the HBM check of source/Task/RicohUtil.cpp:
   1135-1170).  max_batch: frames per scheduling tick. */
int ps_server_create(long long budget_bytes, int max_batch, ps_server** out);
void ps_server_destroy(ps_server* s);
/* Admit a stream whose rig is described like ps_render_prepare.  Returns
   PS_ENOMEM (nothing admitted) when its resident bytes would exceed the
   budget.  *stream_id receives the id. */
int ps_server_admit(ps_server* s, const ps_photo_param* params, int num_params, int blend_param, int src_w,
                    int src_h, int dst_w, int dst_h, int* stream_id);
int ps_server_remove(ps_server* s, int stream_id);
long long ps_server_resident_bytes(const ps_server* s);
/* Replay an arrival trace in real time: frame k of the trace arrives at
   arrival_ns[k] (relative to the start) for stream stream_ids[k], with
   camera frames srcs[k] (host BGR32, pinned preferred) and luts[k]
   (num*3*256 or NULL); outputs go to dsts[k] (host BGR32) or nowhere when
   dsts is NULL.  Blocks until every frame is done, then fills
   latency_ns[k] (arrival -> output ready) and *wall_ns. */
int ps_server_run_trace(ps_server* s, int num_frames, const int* stream_ids, const long long* arrival_ns,
                        const ps_image* const* srcs, const uint8_t* const* luts, ps_image* dsts,
                        long long* latency_ns, long long* wall_ns);

#ifdef __cplusplus
}
#endif
#endif /* PANOSTITCH_H */
