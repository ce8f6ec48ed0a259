/*
 * ps_oracle.h -- CPU restatement of PanoStitcher's per-frame stitch path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product path in panostitcher_gb300/ is compared against; the product never
 * links, loads or calls it.  It is also the timed CPU baseline of bench.py.
 *
 * Parity status: PINNED against the reference's own code.  oracle/Makefile's
 * `ref` target compiles the reference's geometry and CPU remap
 * (source/Warp/Remap.cpp, ZReproject.cpp), its integer pyramid kernels and
 * wrappers (source/CudaAccel/CudaPyramid2.cu) and its YUV conversions
 * (source/CudaAccel/ImageProc.cu) unchanged into oracle/_ref/, against a
 * small OpenCV subset and a CPU emulation of the CUDA runtime
 * (oracle/ref/).  Every function below restates the cited reference code in
 * its integer / double semantics and matches that build bit for bit
 * (tests/test_ref_pin.py), except the documented right-edge tap of the
 * bilinear remap; the fixtures in tests/golden/ are that build's outputs.
 * Not pinned (no reference code to build): the LUT formula (getLUT, in a
 * file that needs the exposure solvers), the distance-transform seams
 * (OpenCV's distanceTransform), the linear-blend weights (OpenCV's Gaussian
 * filter) and the nearest-optical-axis seam rule (the benchmark's own rule).
 *
 * Conventions
 *   - images are tightly packed row-major; 4-channel int16/int32 images store
 *     B,G,R,X per pixel (X = channel 3, undefined in the reference and 0 here);
 *   - masks are uint8 0 / 255;
 *   - "level" j has size W_j = (W_{j-1}+1)/2, H_j = (H_{j-1}+1)/2.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PhotoParam (source/Warp/ZReproject.h:17-50), same field order. */
typedef struct orc_param {
    int imageType, cropMode, cropX, cropY, cropWidth, cropHeight;
    int circleX, circleY, circleR;
    double hfov, vfov, alpha, beta, gamma, shiftX, shiftY, shearX, shearY;
    double yaw, pitch, roll;
} orc_param;

/* Remap (source/Warp/ZReproject.h:91-120). */
typedef struct orc_remap {
    int srcImageType;
    double srcTX, srcTY, destTX, destTY;
    double scale[2], shear[2], rot[2], rad[6], mt[3][3];
    double distance, horizontal, vertical;
} orc_remap;

/* ---- geometry ---------------------------------------------------------- */
void orc_remap_init(const orc_param* p, int canvasW, int canvasH, int camW, int camH, orc_remap* r);
void orc_remap_point(const orc_remap* r, double cx, double cy, double* sx, double* sy);
double orc_remap_axis_angle(const orc_remap* r, double cx, double cy);
void orc_reproject_map(const orc_param* p, int camW, int camH, int canvasW, int canvasH,
                       double* map64 /* nullable, 2 per px */, float* xmap, float* ymap, uint8_t* mask);
void orc_nearest_axis_seams(const orc_param* params, int n, int camW, int camH, int canvasW, int canvasH,
                            const uint8_t* coverage /* n*W*H */, uint8_t* seams /* n*W*H */);
/* the same two on canvas rows [row0, row1) only (full-canvas buffers), so
   that callers can split a canvas across threads */
void orc_reproject_map_rows(const orc_param* p, int camW, int camH, int canvasW, int canvasH, int row0, int row1,
                            double* map64, float* xmap, float* ymap, uint8_t* mask);
void orc_nearest_axis_seams_rows(const orc_param* params, int n, int camW, int camH, int canvasW, int canvasH,
                                 int row0, int row1, const uint8_t* coverage, uint8_t* seams);
void orc_get_lut(double k, uint8_t lut[256]);

/* ---- remap ------------------------------------------------------------- */
void orc_reproject_bilinear_16s(const uint8_t* src, int srcW, int srcH, long long srcStep, int channels,
                                const uint8_t* lut /* 3*256 (B,G,R) or NULL */,
                                const float* xmap, const float* ymap, int dstW, int dstH,
                                int16_t* dst /* dstW*dstH*4 */);
void orc_reproject_bilinear_16s_rows(const uint8_t* src, int srcW, int srcH, long long srcStep, int channels,
                                     const uint8_t* lutted /* unused when NULL */, const float* xmap, const float* ymap,
                                     int dstW, int row0, int row1, int16_t* dst);

/* ---- pyramid primitives (CudaAccel/CudaPyramid2.cu semantics) ----------- */
int orc_num_levels(int width, int height, int maxLevels, int minLength);
void orc_level_sizes(int w, int h, int levels, int* ws, int* hs);
void orc_pyr_down_16sc1_to_32sc1(const int16_t* src, int sw, int sh, int32_t* dst, int dw, int dh);
void orc_pyr_down_16sc1_to_16sc1(const int16_t* src, int sw, int sh, int16_t* dst, int dw, int dh);
void orc_pyr_down_16sc4_masked(const int16_t* src, int sw, int sh, const int32_t* scale,
                               int16_t* dst, int dw, int dh);
void orc_pyr_up_16sc4(const int16_t* src, int sw, int sh, int16_t* dst, int dw, int dh);
void orc_pyr_up_32sc4(const int32_t* src, int sw, int sh, int32_t* dst, int dw, int dh);

/* ---- multiband blend (CudaTilingMultibandBlendFast semantics) ----------- */
typedef struct orc_blender orc_blender;
orc_blender* orc_mb_prepare(const uint8_t* masks /* n*W*H coverage */, const uint8_t* seams /* n*W*H */,
                            int n, int W, int H, int maxLevels, int minLength);
void orc_mb_free(orc_blender* b);
/* blend(images, masks, blendImage) (CudaMultibandBlend.cpp:825-893): later
   blends take their weights from the n*W*H custom masks, normalise by the
   weight sums whatever the coverage and zero the pixels outside the masks'
   union; masks = NULL restores the prepared unique masks. */
int orc_mb_set_custom_masks(orc_blender* b, const uint8_t* masks);
int orc_mb_num_levels(const orc_blender* b);
int orc_mb_full_mask(const orc_blender* b);
/* copies of prepared pyramids for bit-exact checks */
void orc_mb_get_alpha(const orc_blender* b, int cam, int level, int32_t* out);
void orc_mb_get_weight(const orc_blender* b, int cam, int level, int16_t* out);
/* blend of n int16x4 level-0 images (each W*H*4) into BGR32 (W*H*4, X=0).
   If level_out != NULL it receives the normalised (pre-collapse) int32x4
   pyramid followed by the collapsed pyramid, level by level. */
void orc_mb_blend(orc_blender* b, const int16_t* const* images, uint8_t* dst, int32_t* norm_out, int32_t* coll_out);
/* same arithmetic, camera pyramids built on nthreads threads */
void orc_mb_blend_mt(orc_blender* b, const int16_t* const* images, uint8_t* dst, int nthreads);

/* ---- multiband blend, CPU semantics (TilingMultibandBlendFast) ------------ */
/* The reference's CPU twin of the blend (source/Blend/MultiBandBlend.cpp:
   906-1031 with source/Blend/Pyramid.cpp), restated in ps_oracle_cpu.c.  It
   differs from the CudaAccel semantics above, which the product computes:
   the masked pyrDown divides ((S << 8) - S) by the alpha sum, the full-mask
   normalisation is R >> 8, the Laplacian subtract saturates, and its borders
   are OpenCV's (reflect-101 rows, wrapped columns).  Same inputs as
   orc_mb_prepare: coverage masks and unique masks, n*W*H each.  coll_out
   (nullable) receives the collapsed result pyramid, int32x3 per pixel,
   levels 0..L packed.  nthreads host threads; the result does not depend on
   them. */
typedef struct orc_cpu_blender orc_cpu_blender;
orc_cpu_blender* orc_cpu_mb_prepare(const uint8_t* masks, const uint8_t* seams, int n, int W, int H, int maxLevels,
                                    int minLength);
void orc_cpu_mb_free(orc_cpu_blender* b);
int orc_cpu_mb_num_levels(const orc_cpu_blender* b);
int orc_cpu_mb_full_mask(const orc_cpu_blender* b);
void orc_cpu_mb_get_weight(const orc_cpu_blender* b, int cam, int level, int16_t* out);
void orc_cpu_mb_get_alpha(const orc_cpu_blender* b, int cam, int level, int32_t* out);
void orc_cpu_mb_blend(orc_cpu_blender* b, const int16_t* const* images, uint8_t* dst, int32_t* coll_out,
                      int nthreads);
/* CPUPanoramaRender::render (source/Task/RicohUtil.cpp:1481-1587): per camera
   LUT, row-parallel bilinear remap to int16, then the CPU blend; arguments as
   orc_render. */
void orc_cpu_render(orc_cpu_blender* b, const uint8_t* const* srcs, int srcW, int srcH, int channels,
                    const uint8_t* luts, const float* const* xmaps, const float* const* ymaps, uint8_t* dst,
                    int nthreads);

/* ---- whole render (CPUPanoramaRender / CudaPanoramaRender2 dataflow) ---- */
/* srcs: n BGR24/BGR32 frames; luts: n*3*256 or NULL; maps: n float x/y maps.
   Writes BGR32 dst.  nthreads>1 uses the row-parallel remap and the
   camera-parallel blend. */
void orc_render(orc_blender* b, const uint8_t* const* srcs, int srcW, int srcH, int channels,
                const uint8_t* luts, const float* const* xmaps, const float* const* ymaps,
                uint8_t* dst, int nthreads);

/* ---- reference seams: getNonIntersectingMasks (source/Blend/Mask.cpp:376-398) */
/* L1 distance of every pixel of an 8-bit mask to its nearest zero pixel, by
   the two-pass 3x3 chamfer with unit horizontal / vertical and diagonal 2
   steps (cv::distanceTransform(src, dst, CV_DIST_L1, 3)); pixels outside
   the image are not zeros.  A mask without any zero pixel gets ORC_DT_FAR
   plus the chamfer distance to the image border everywhere. */
#define ORC_DT_FAR (1 << 28)
void orc_distance_transform_l1(const uint8_t* mask, int W, int H, int32_t* dist);
/* masks: n W*H 0/non-zero coverage masks; out: n W*H 0/255 unique masks. */
void orc_non_intersecting_masks(const uint8_t* masks, int n, int W, int H, uint8_t* out);

/* ---- linear blend (highQualityBlend == 0) -------------------------------- */
/* getWeightsLinearBlend32F (source/Blend/LinearBlend.cpp:136-151) over given
   coverage and unique masks (n W*H each, 0/non-zero): Gaussian blur of
   radius r (2r+1 taps, sigma r/3, reflect-101) of each unique mask in 8-bit
   fixed point, AND coverage, then calcWeights32F (:78-120).  weights: n W*H
   floats. */
void orc_linear_weights(const uint8_t* coverage, const uint8_t* seams, int n, int W, int H, int r, float* weights);
/* The linear-blend render: per camera LUT + double bilinear remap to bytes,
   then accum += byte * weight in fp32 in camera order, then round half to
   even and saturate (RicohUtil.cpp:1269-1286 with the CPU
   reprojectWeightedAccumulateTo32F, source/Warp/ZReproject.cpp:606-633).
   Writes BGR32 dst (W*H*4). */
void orc_linear_render(const uint8_t* const* srcs, int srcW, int srcH, int channels, const uint8_t* luts,
                       const float* const* xmaps, const float* const* ymaps, const float* weights, int n, int W,
                       int H, uint8_t* dst);

/* ---- encoder handoff --------------------------------------------------- */
/* cvtBGR32ToYUV420P / cvtBGR32ToNV12 (source/CudaAccel/ImageProc.cu:44-160):
   BT.601 studio range in 20-bit fixed point.  fmt 420: planes y, u, v;
   fmt 12 (NV12): planes y, uv (v unused).  w, h even. */
void orc_bgr32_to_yuv(const uint8_t* bgr, long long bgrStep, int w, int h, int fmt, uint8_t* y, long long yStep,
                      uint8_t* u, long long uStep, uint8_t* v, long long vStep);
/* cvtYUV420PToBGR32 / cvtNV12ToBGR32 (source/CudaAccel/ImageProc.cu:165-222):
   planes y, u, v (fmt 420) or y, uv (fmt 12) of an even-sized frame to
   BGR32 (fourth byte 0). */
void orc_yuv_to_bgr32(const uint8_t* y, long long yStep, const uint8_t* u, long long uStep, const uint8_t* v,
                      long long vStep, int w, int h, int fmt, uint8_t* bgr, long long bgrStep);

#ifdef __cplusplus
}
#endif
#endif
