// ps_internal.h -- host-side internals shared by the library's translation units.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "ps_device.cuh"

namespace ps {

// An NVTX range over a scope of host code (prepare, each render run, the
// autotuner, each launch issued outside a graph), so a profiler's timeline
// shows the library's phases beside the kernels.  NVTX calls cost nothing
// measurable unless a tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---- errors -------------------------------------------------------------------
// Internal code throws ps::Error; the C ABI converts it to a status code and
// the thread-local message returned by ps_last_error().
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char* fmt, ...);
void setLastError(const std::string& msg);  // the text ps_last_error() returns
void checkCuda(cudaError_t e, const char* what);
#define PS_CUDA(call) ::ps::checkCuda((call), #call)

// ---- device memory --------------------------------------------------------------
// Owning device allocation; every allocation of the library goes through it
// so resident bytes can be accounted for admission control.
class DevBuf {
public:
    DevBuf() = default;
    explicit DevBuf(size_t bytes) { alloc(bytes); }
    ~DevBuf() { reset(); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o) { reset(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
        return *this;
    }
    void alloc(size_t bytes);
    void reset();
    void zero(cudaStream_t st);
    template <class T> T* as() const { return static_cast<T*>(p_); }
    void* get() const { return p_; }
    size_t bytes() const { return n_; }

private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// Pinned host allocation.
class HostBuf {
public:
    HostBuf() = default;
    ~HostBuf() { reset(); }
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    void alloc(size_t bytes);
    void reset();
    template <class T> T* as() const { return static_cast<T*>(p_); }
    size_t bytes() const { return n_; }

private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// ---- geometry -------------------------------------------------------------------
// Remap (source/Warp/ZReproject.h:91-120) after init, flattened for the GPU.
struct RemapDev {
    int type;                      // PanoTools source type: 0 rectilinear, 2 circular, 3 full-frame fisheye
    double srcTX, srcTY, destTX, destTY;
    double scale0, scale1, shear0, shear1, rot0, rot1;
    double rad[6];
    double mt[9];
    double distance, horizontal, vertical;
    // validity test of getReprojectMapAndMask (source/Warp/ZReproject.cpp:132-219)
    int camW, camH;
    int circ;                      // image types 2 / 3: crop rectangle and circle
    int cropX, cropY, cropW, cropH;
    double centx, centy, sqrDist;
};

void remapInit(const ps_photo_param& p, int canvasW, int canvasH, int camW, int camH, RemapDev& out);
int trueNumLevels(int width, int height, int maxLevels, int minLength);

cudaError_t launchGenMap(const RemapDev* dParam, int W, int H, float* xmap, float* ymap, uint8_t* cov,
                         cudaStream_t st);
cudaError_t launchNearestAxisSeams(const RemapDev* dParams, int n, int W, int H, const uint8_t* cov,
                                   uint8_t* seams, cudaStream_t st);
// getNonIntersectingMasks: n W*H coverage masks -> n 0/255 unique masks.
// Scratch: uni W*H bytes, dUni and dCam W*H int32 each.
cudaError_t launchNonIntersectingMasks(const uint8_t* cov, int n, int W, int H, uint8_t* out, uint8_t* uni,
                                       int32_t* dUni, int32_t* dCam, cudaStream_t st);
// Linear-blend weights of n cameras (taps: 2r+1 fixed-point Gaussian taps on
// the device), full-canvas into wFull and tile-compact (items) into wCompact.
// Scratch: rowsScratch n*W*H int32, distScratch n*W*H bytes.
cudaError_t launchLinearWeights(const uint8_t* seam, const uint8_t* cov, int n, int W, int H, const int* taps, int r,
                                int32_t* rowsScratch, uint8_t* distScratch, float* wFull, const RemapItem* items,
                                int nitems, float* wCompact, cudaStream_t st);
// exact L1 distance of every pixel to the nearest zero pixel (>= 2^28 when there is none)
cudaError_t launchDistanceTransformL1(const uint8_t* mask, int W, int H, int32_t* dist, cudaStream_t st);

// ---- prepare-time pyramids --------------------------------------------------------
// level 0: Wt = seam ? 256 : 0, A (0/256 scratch) = cov ? 256 : 0
cudaError_t launchInitLevel0(const uint8_t* cov, const uint8_t* seams, int W, int H, long long maskStride,
                             uint16_t* wt, uint16_t* a0, int pitch, long long camStride, int n,
                             cudaStream_t st);
// alpha chain: raw = pyrDown16SC1To32SC1(a_j); am = raw >> 8; a_{j+1} = raw ? 256 : 0
cudaError_t launchAlphaDown(const uint16_t* aj, int sw, int sh, int spitch, long long sstride, uint16_t* am,
                            uint16_t* anext, int dw, int dh, int dpitch, long long dstride, int n,
                            cudaStream_t st);
// weight chain: Wt_{j+1} = (pyrDown(Wt_j) + 128) >> 8
cudaError_t launchWeightDown(const uint16_t* wj, int sw, int sh, int spitch, long long sstride, uint16_t* wn,
                             int dw, int dh, int dpitch, long long dstride, int n, cudaStream_t st);
// per-tile "any non-zero" flags of a 16-bit or 8-bit plane per camera
cudaError_t launchTileFlags16(const uint16_t* p, int w, int h, int pitch, long long camStride, int n, int tw,
                              int th, int tilesX, int tilesY, uint8_t* flags, cudaStream_t st);
cudaError_t launchTileNot256(const uint16_t* p, int w, int h, int pitch, long long camStride, int n, int tw, int th,
                             int tilesX, int tilesY, uint8_t* flags, cudaStream_t st);
cudaError_t launchTileFlags8(const uint8_t* p, int w, int h, int pitch, long long camStride, int n, int tw,
                             int th, int tilesX, int tilesY, uint8_t* flags, cudaStream_t st);
// number of non-zero pixels of a 16-bit plane, all cameras (added to *out)
cudaError_t launchCountNonzero16(const uint16_t* p, int w, int h, int pitch, long long camStride, int n,
                                 unsigned long long* out, cudaStream_t st);
// union coverage (0/255) and per-tile covered-pixel counts
cudaError_t launchUnion(const uint8_t* cov, int n, int W, int H, long long maskStride, uint8_t* uni, int pitch,
                        int tw, int th, int tilesX, int* tileCounts, unsigned long long* total,
                        cudaStream_t st);
// copy full-canvas maps into tile-compact float2 storage
// map-free remap: coverage bits per remap tile (16 words each, map-tile
// order) and the fp32 parameters of a camera
cudaError_t launchCovTiles(const uint8_t* cov, int W, int H, long long maskStride, const RemapItem* items,
                           int nitems, uint32_t* words, cudaStream_t st);
RemapParamF remapParamF(const RemapDev& r);
cudaError_t launchCompactMaps(const float* xmap, const float* ymap, int W, int H, long long maskStride,
                              const RemapItem* items, int nitems, float2* maps, cudaStream_t st);
// int16x4 / uint8x4 images -> uchar4 level 0, checking range and zero outside coverage
cudaError_t launchImagesToLevel0(const void* const* images, const long long* pitches, int fmt, int n, int W,
                                 int H, const uint8_t* cov, long long maskStride, uchar4* g0, int pitch,
                                 long long camStride, int* status, cudaStream_t st);

// ---- launch shapes ----------------------------------------------------------------
// The launch choices that can change after prepare.  Tile sizes are fixed
// at compile time (the tile-compact maps and the 2x2 blend layout depend on
// them); what varies is which levels the tail kernel runs, its cluster
// width and tile split, and the CTAs per SM of the persistent kernels.
// Set by hand or chosen by the autotuner (ps_tune.cpp).
struct LaunchShape {
    int tailMaxItems = 16;         // levels with at most this many tiles run in the tail kernel (0: none)
    int tailCluster = 0;           // CTAs per rig in the tail kernel: 8, 16, or 0 = the widest co-schedulable
    int tailHalf = 1;              // the tail blends levels above 0 in 64x8 half tiles
    int ctasPerSm[3] = {0, 0, 0};  // k_remap, k_pyrdown, k_blend; 0 = as many as fit
    int smallBlendMaxItems = 0;    // blend levels above 0 with at most this many tiles run in k_blend_small
    int remapDefer = 1;            // near-tie remap pixels recomputed by k_remap_fix (1) or inside k_remap (0)
    bool operator==(const LaunchShape& o) const
    {
        return tailMaxItems == o.tailMaxItems && tailCluster == o.tailCluster && tailHalf == o.tailHalf &&
               ctasPerSm[0] == o.ctasPerSm[0] && ctasPerSm[1] == o.ctasPerSm[1] && ctasPerSm[2] == o.ctasPerSm[2] &&
               smallBlendMaxItems == o.smallBlendMaxItems && remapDefer == o.remapDefer;
    }
    bool operator!=(const LaunchShape& o) const { return !(*this == o); }
};

// ---- per-frame kernels ------------------------------------------------------------
// perSm > 0 caps the CTAs per SM of the one-wave persistent grid; counter
// (remap and blend) is a zeroed int through which the launch hands out its
// work items
// defer: near-tie pixels go on the list (tieCount, ties) for launchRemapFix;
// otherwise k_remap recomputes them itself.  srcFmt: the format of every
// source of the launch (PS_FMT_BGR32 selects the specialised kernel), or 0
// when they differ
cudaError_t launchRemap(const Segment* segs, int nsegs, int total, int perSm, int* counter, int* tieCount,
                        RemapTie* ties, bool defer, int srcFmt, cudaStream_t st);
// the pixels k_remap listed as lying near a rounding tie, recomputed exactly;
// ties has room for kRemapTiesPerTile entries per remap tile of the launch,
// and tieCount is a zeroed int
cudaError_t launchRemapFix(const Segment* segs, int nsegs, int total, const int* tieCount, const RemapTie* ties,
                           cudaStream_t st);
constexpr int kRemapTiesPerTile = 2;
cudaError_t launchPyrDown(const Segment* segs, int nsegs, int total, int perSm, cudaStream_t st);
// counter: a zeroed int the launch hands its tiles out through
// Accesses the checked build's kernels refused since the last reset
// (waits for the device); -1 in the normal build, -2 on a CUDA error.
long long boundsViolations(bool reset);
// probePolls > 0: the failure-path test of the bounded waits (k_blend).
// early: the launch before this one wrote only C levels (a blend step after
// the first), so the G_j, weight and G_{j+1} reads of each CTA's first unit
// may be issued before the wait for it (k_blend, k_blend_small)
cudaError_t launchBlend(const Segment* segs, int nsegs, int total, int perSm, int* counter, int probePolls,
                        bool early, cudaStream_t st);
// blend of few-tile levels above 0: two work items (the 64x8 halves) per tile
cudaError_t launchBlendSmall(const Segment* segs, int nsegs, int total, bool early, cudaStream_t st);
// one cluster per segment: the rig's pyrDown levels tailDown..L and blend
// levels L..tailBlend; cluster 8 or 16 CTAs (0 or more than the GPU
// co-schedules: the widest it does)
cudaError_t launchTail(const Segment* segs, int nsegs, int cluster, cudaStream_t st);
// CTAs of k_remap (kind 0), k_pyrdown (1), k_blend (2) resident per SM;
// the widest tail cluster the GPU co-schedules (8 or 16)
int residentCtasPerSm(int kind);
int tailClusterMax();
// linear-blend mode: LinearItems of every segment; maxCams sizes the LUT stage
cudaError_t launchLinear(const Segment* segs, int nsegs, int total, int maxCams, cudaStream_t st);

// ---- camera parameter files (ps_params.cpp) ----------------------------------------
// loadPhotoParams for PTGui .pts files; empty when the file holds no usable
// cameras; throws PS_EINVAL for other file types or an unreadable file.
std::vector<ps_photo_param> loadPhotoParams(const std::string& path);

// ---- standalone primitives -------------------------------------------------------
cudaError_t launchReprojectTo16S(const uint8_t* src, long long srcPitch, int srcW, int srcH, int srcFmt,
                                 const float* xmap, const float* ymap, long long mapPitch, int dstW, int dstH,
                                 const uint8_t* lut, int16_t* dst, long long dstPitch, cudaStream_t st);
// YUV420P / NV12 frames -> BGR32 (one launch for all f.n frames)
cudaError_t launchYuvToBgr32(const YuvFrames& f, cudaStream_t st);
// BGR32 -> YUV420P (u, v planes) or NV12 (u = the UV plane, v unused); w, h even
cudaError_t launchCvtYuv(const uint8_t* src, long long srcPitch, int w, int h, int fmt, uint8_t* y, long long yPitch,
                         uint8_t* u, long long uPitch, uint8_t* v, long long vPitch, cudaStream_t st);

}  // namespace ps
