// ps_device.cuh -- device-side data layout shared by the stitch kernels.
//
// HBM layout of one rig (all cameras share the level geometry):
//   G[j]   uchar4 Gaussian pyramid of every camera, level j, camera-major,
//          row pitch lv[j].pitch pixels.  The reference keeps it as int16x4
//          (CV_16SC4); every value is provably in 0..255 (the level-0 remap
//          is a convex combination of bytes and each masked pyrDown is a
//          weighted average of the level below), so one byte per channel is
//          exact and halves the traffic.
//   Wt[j]  uint16 seam-weight pyramid (weightPyrs, 0..256), same pitch as G.
//   Am[j]  uint16 alpha divisor m = alphaPyr / 256 (alphaPyrs is always a
//          multiple of 256 because its level source is 0/256), level >= 1.
//   C[j]   short4 collapsed result of level j >= 1 (resultPyr after
//          normalise + collapse); |value| < 3300 so int16 is exact.
//   maps   float2 dst->src map, stored tile-compact for the level-0 tiles
//          that a camera covers (512 pixels per 32x16 tile, row-major in the tile).
// Work is described by item lists built at prepare time from the pyramids'
// supports, so no kernel touches canvas area a camera cannot influence.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/panostitch.h"

namespace ps {

// ---- tiles ------------------------------------------------------------------
constexpr int kRemapTW = 32, kRemapTH = 16;    // level-0 remap tile (two pixels per thread)
constexpr int kDownTW = 32, kDownTH = 16;      // pyrDown output tile (two pixels per thread)
constexpr int kBlendTW = 64, kBlendTH = 16;    // blend tile (a 2x2 pixel block per thread)
constexpr int kThreads = 256;

struct LevelDev {
    int w, h;            // level size
    int pitch;           // row pitch in pixels of G / Wt / Am / C (multiple of 64)
    long long camStride; // pixels between cameras in G / Wt / Am
    uchar4* G;
    uint16_t* Wt;
    uint16_t* Am;
    short4* C;
};

// Work items (one per tile), resident per rig and built at prepare time.
struct RemapItem { uint16_t cam, pad; uint16_t tx, ty; uint32_t mapTile; };

struct DownItem { uint8_t cam, level; uint16_t tx, ty; uint16_t pad; };   // level = output level
// A blend tile lists the cameras whose weight touches it: up to 8 inline,
// more through RigDev::camLists (cams[0..3] then hold the uint32 offset).
struct alignas(16) BlendItem { uint8_t level, cls, camCnt, flags; uint16_t tx, ty; uint8_t cams[8]; };
constexpr int kInlineCams = 8;
// flags bit 0: one camera, weight 256 on every pixel of the tile, so the
// normalised value is the Laplacian itself (R = 256 L, W = 256).
constexpr int kTileUniform = 1;
// cls of a level-0 blend tile: 0 uncovered (write zeros), 1 fully covered,
// 2 partially covered (read the union mask).  Unused above level 0.
// Linear-blend mode: one item per 32x16 canvas tile, naming the run
// [first, first + count) of remap items (cameras in index order) covering it.
struct LinearItem { uint16_t tx, ty; uint32_t first, count; };

// Remap::remapImage's parameters in fp32, for the map-free remap (the
// reference's dstToSrc, source/CudaAccel/CudaReproject.cu:81-264, keeps them
// in double).
struct RemapParamF {
    int type;  // 0 rectilinear, else fisheye
    float srcTX, srcTY, destTX, destTY;
    float scale0, scale1, shear0, shear1, rot0, rot1;
    float rad[6];
    float mt[9];
    float distance, horizontal, vertical;
};

// The tensor maps of one level for k_blend's producer (boxes of the bulk
// tensor copies): the level's G tile (64 x 16 x 1 of uint32 over pitch x h x
// cameras), its G footprint as the level above a blend (40 x 10 x 1), its
// collapsed C footprint (36 x 10 of 8-byte pixels over pitch x h) and its
// weight tile (64 x 16 x 1 of uint16).
constexpr int kTmG = 0, kTmGfp = 1, kTmC = 2, kTmW = 3, kTmapsPerLevel = 4;

struct RigDev {
    int n, L, W, H;
    int full;                 // union of coverages == whole canvas
    int srcW, srcH;
    const float2* maps;       // tile-compact maps of all cameras (NULL when map-free)
    int numRemapItems;        // tiles of the maps (and of the map-free coverage words)
    // map-free remap: per camera its parameters, per remap tile (in map-tile
    // order) its coverage as 16 words of 32 bits, one word per tile row
    const RemapParamF* camsF;
    const uint32_t* covTiles;
    const uint8_t* unionMask; // level-0 union coverage (0/255), pitch = lv[0].pitch
    const uint8_t* camLists;  // camera indices of blend tiles with more than 8 cameras
    // TMA tensor maps of this state slot (CUtensorMap, 128 bytes each, 64-byte
    // aligned in device memory), kTmapsPerLevel per level: see kTmG ... kTmW;
    // NULL when they could not be encoded (k_blend then copies row by row)
    const void* tmaps;
    LevelDev lv[PS_MAX_LEVELS + 1];
    // work items of every level (used by the tail kernel)
    const DownItem* downItems;
    const BlendItem* blendItems;
    int downOff[PS_MAX_LEVELS + 1], downCnt[PS_MAX_LEVELS + 1];
    int blendOff[PS_MAX_LEVELS + 1], blendCnt[PS_MAX_LEVELS + 1];
    // the small top of the pyramid runs in one launch: pyrDown levels
    // tailDown..L, then blend levels L..tailBlend (L + 1 = none); with
    // tailHalf the blend levels above 0 go in 64x8 half tiles
    int tailDown, tailBlend, tailHalf;
    // linear-blend mode: the remap items (tile-major) and their weights,
    // 512 floats per item in the layout of the maps
    const RemapItem* remapItems;
    const float* linWeights;
};

// Per-frame arguments of one rig in a launch (device resident, rewritten
// before every launch sequence).
struct FrameDev {
    const uint8_t* src[PS_MAX_CAMS];
    long long srcPitch[PS_MAX_CAMS];
    int srcFmt;               // PS_FMT_BGR24 / PS_FMT_BGR32
    int outFmt;               // PS_FMT_BGR24 / BGR32 / YUV420P / NV12
    uint8_t* out;             // BGR canvas, or the Y plane
    long long outPitch;
    uint8_t* outU;            // YUV420P: U plane; NV12: interleaved UV plane
    uint8_t* outV;            // YUV420P: V plane
    long long outCPitch;      // pitch of the U (or UV) plane
    long long outVPitch;      // pitch of the V plane
    const uint8_t* luts;      // n * 768 device bytes (B, G, R tables)
    int* status;              // device error word (0 = ok)
};

// Decoder frames to convert to BGR32 (k_yuv_to_bgr32): YUV420P (u, v
// planes) or NV12 (u = the interleaved UV plane), all w x h (even).
struct YuvFrame {
    const uint8_t *y, *u, *v;
    long long yPitch, uPitch, vPitch;
    uint8_t* dst;
    long long dstPitch;
    int fmt;
    int vec;  // w % 8 == 0 and every plane aligned for 8-pixel-wide vector access
};
struct YuvFrames {
    YuvFrame frame[PS_MAX_CAMS];
    int n, w, h;
};

// A launch runs the concatenation of segments: `count` items of one rig,
// numbered from `prefix` in the launch.  Several rigs (a batch, or the
// frames of a serving tick) share one launch this way.
struct Segment {
    const void* items;
    const RigDev* rig;
    const FrameDev* frame;
    int count, prefix;
};

// A level-0 pixel whose fp32 remap lies near a rounding tie, listed by the
// remap for its exact recompute: everything the recompute needs without
// looking the tile up again.
struct RemapTie {
    const FrameDev* frame;
    const RigDev* rig;
    float mx, my;    // the map value
    uint32_t pixel;  // y * pitch + x in the camera's level-0 plane
    int cam;
};

#ifdef __CUDACC__
// Item `it` of a launch -> its segment, scanning forward from a hint (each
// CTA visits its items in increasing order).
__device__ __forceinline__ int findSegment(const Segment* segs, int nsegs, int it, int hint)
{
    int s = hint;
    while (s + 1 < nsegs && segs[s + 1].prefix <= it) s++;
    return s;
}

// Contiguous chunk of items for this CTA (k_pyrdown): neighbouring tiles of
// one camera stay on one SM, and no item is handed out through an atomic.
__device__ __forceinline__ void itemRange(int total, int& begin, int& end)
{
    const int chunk = (total + gridDim.x - 1) / gridDim.x;
    begin = min(total, (int)blockIdx.x * chunk);
    end = min(total, begin + chunk);
}


// ---- borders: source/CudaAccel/CudaUtil.cuh:6-98 ------------------------------
// Vertical reflect-101 (BrdColReflect101) and horizontal wrap (BrdRowWrap),
// restated with the reference's exact index formulas.
__device__ __forceinline__ int rowLow(int y, int H) { return abs(y) % H; }
__device__ __forceinline__ int rowHigh(int y, int H) { int last = H - 1; return abs(last - abs(last - y)) % H; }
__device__ __forceinline__ int colLow(int x, int W) { return x >= 0 ? x : x - ((x - W + 1) / W) * W; }
__device__ __forceinline__ int colHigh(int x, int W) { return x < W ? x : x % W; }
// any row index of a pyramid tile -> the row the reference reads
__device__ __forceinline__ int rowMap(int y, int H) { return y < 0 ? rowLow(y, H) : (y >= H ? rowHigh(y, H) : y); }
__device__ __forceinline__ int colMap(int x, int W) { return x < 0 ? colLow(x, W) : (x >= W ? colHigh(x, W) : x); }

// C truncating division a / d given rcp = __frcp_rn(d), exact for |a| < 2^24
// (exact in fp32), 1 <= d < 2^16 and |a| / d < 2^21: the fp32 quotient then
// has a relative error below 2^-22, so it is within 1 of the true one, and one
// remainder check fixes it.  The normalisation divides weighted sums of
// Laplacians by their weight sums: |a| <= 255 d < 2^23, quotients <= 255.
__device__ __forceinline__ int divTrunc(int a, int d, float rcp)
{
    const int m = abs(a);
    int q = (int)__fmul_rz((float)m, rcp);
    const int r = m - q * d;
    q += (r >= d) - (r < 0);
    return a < 0 ? -q : q;
}

// Programmatic dependent launch: wait until the previous kernel in the
// stream has completed and its writes are visible (everything before this
// call may only touch data that kernel does not write).
__device__ __forceinline__ void waitPrevGrid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Let the next kernel in the stream start launching (its CTAs block in
// waitPrevGrid until this grid completes).
__device__ __forceinline__ void allowNextGrid() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// ---- packed channel arithmetic -----------------------------------------------
// A BGRX byte quad splits into two words holding 16-bit lanes:
//   lo = B | R << 16,  hi = G | X << 16.
// Sums of up to 256 weighted bytes stay below 65536, so the 5x5 pyramid
// filters run two channels per 32-bit add with no carry between lanes.
__device__ __forceinline__ uint2 unpackBytes(uint32_t v)
{
    return make_uint2(v & 0x00FF00FFu, (v >> 8) & 0x00FF00FFu);
}
#endif  // __CUDACC__

}  // namespace ps
