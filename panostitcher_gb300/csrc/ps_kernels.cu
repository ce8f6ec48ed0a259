// ps_kernels.cu -- the per-frame stitch kernels (sm_103a).
//
// One frame of one or more rigs runs as about 2L+2 launches over prepared
// work lists:
//   k_remap        level 0: LUT gain + bilinear remap of every covered tile,
//                  written as uchar4 G0 (cudaTransform + cudaReprojectTo16S);
//   k_remap_fix    (launch shapes that defer them) the near-tie pixels the
//                  remap listed, recomputed with the double sequence;
//   k_pyrdown      levels 1..L: masked 5x5 decimation G_j -> G_{j+1}
//                  (pyrDown16SC4To16SC4 with alpha scale);
//   k_blend        levels L..0: for every canvas tile, the Laplacian of each
//                  camera whose seam weight touches the tile
//                  (G_j - pyrUp(G_{j+1})), its weighted accumulation, the
//                  normalisation, and the collapse step pyrUp(C_{j+1}) + N_j,
//                  all in registers; level 0 writes the 8-bit output with
//                  the uncovered pixels zeroed;
//   k_blend_small, k_tail  the same for the few-tile top levels (half tiles;
//                  one thread-block cluster running several levels).
// The reference runs the same arithmetic as ~35 launches per camera plus
// ~36 per frame over full-canvas int16/int32 images
// (source/CudaAccel/CudaMultibandBlend.cpp:785-823).
#include <algorithm>
#include <cstddef>
#include <cstdlib>

#include "ps_async.cuh"
#include "ps_device.cuh"
#include "ps_internal.h"

namespace ps {

__constant__ int c_k5[5] = {1, 4, 6, 4, 1};

// ---- the checked build ---------------------------------------------------------
// Compiled with -DPS_CHECK_BOUNDS (libpanostitch_checked.so), every global
// access of the stitch kernels is checked against the extent of the buffer
// it belongs to.  An access outside is not made -- a load reads 0, a store
// is dropped, a bulk copy reads from the buffer's start instead, so its
// byte count still completes its barrier -- and the device-wide violation
// counter goes up (ps_debug_bounds_violations).  Nothing traps.  In the
// normal build every check is a constant true.
#ifdef PS_CHECK_BOUNDS
__device__ unsigned long long g_boundsViolations;
#endif

template <class T>
__device__ __forceinline__ bool inside(const T* p, const void* base, long long bytes)
{
#ifdef PS_CHECK_BOUNDS
    const char* c = reinterpret_cast<const char*>(p);
    const char* b = static_cast<const char*>(base);
    if (!base || c < b || c + sizeof(T) > b + bytes) {
        atomicAdd(&g_boundsViolations, 1ull);
        return false;
    }
#endif
    return true;
}

// [p, p + n) inside [base, base + bytes)
__device__ __forceinline__ bool insideRange(const void* p, long long n, const void* base, long long bytes)
{
#ifdef PS_CHECK_BOUNDS
    const char* c = static_cast<const char*>(p);
    const char* b = static_cast<const char*>(base);
    if (!base || c < b || c + n > b + bytes) {
        atomicAdd(&g_boundsViolations, 1ull);
        return false;
    }
#endif
    return true;
}

template <class T>
__device__ __forceinline__ T ldChecked(const T* p, const void* base, long long bytes)
{
    return inside(p, base, bytes) ? __ldg(p) : T{};
}

// A bulk copy whose source range is checked: outside its buffer it copies
// from the buffer's start instead, so the barrier still receives its bytes.
__device__ __forceinline__ void bulkCopyChecked(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                const void* base, long long ext)
{
    if (!insideRange(src, bytes, base, ext)) src = base;
    bulkCopy(dst, src, bytes, bar);
}

// Extents of a rig's buffers.
__device__ __forceinline__ long long gBytes(const RigDev& R, const LevelDev& L) { return (long long)R.n * L.camStride * 4; }
__device__ __forceinline__ long long wBytes(const RigDev& R, const LevelDev& L) { return (long long)R.n * L.camStride * 2; }
__device__ __forceinline__ long long cBytes(const LevelDev& L) { return (long long)L.pitch * L.h * 8; }

// ============================================================================
// Remap of one canvas pixel: cudaTransform (source/CudaAccel/
// CudaGainAdjust.cu:57-101) fused with the bilinear map remap.  The
// arithmetic follows the double-precision CPU bilinear (source/Warp/
// ZReproject.cpp:101-130): weights from the float map coordinates, taps
// (x0,y0) (x1,y0) (x0,y1) (x1,y1) with x1 and y1 clamped to the frame, the
// result rounded half to even.  The fast path computes in fp32 (absolute
// error < 1.3e-4 for values <= 255); a result within 2e-4 of a rounding tie
// is recomputed with the reference's exact sequence of IEEE double
// operations, so the stored byte equals the double-precision one.
// ============================================================================
__device__ __forceinline__ uint32_t loadTexel(const uint8_t* row, int x, int fmt, const uint8_t* base, long long bytes)
{
    if (fmt == PS_FMT_BGR32) return ldChecked(reinterpret_cast<const uint32_t*>(row) + x, base, bytes);
    const uint8_t* p = row + 3 * x;
    if (!insideRange(p, 3, base, bytes)) return 0;
    return (uint32_t)__ldg(p) | ((uint32_t)__ldg(p + 1) << 8) | ((uint32_t)__ldg(p + 2) << 16);
}

__device__ __noinline__ int bilinearExact(double x, double y, int x0, int y0, int p00, int p01, int p10, int p11)
{
    const double wx0 = __dsub_rn(x, (double)x0), wx1 = __dsub_rn(1.0, wx0);
    const double wy0 = __dsub_rn(y, (double)y0), wy1 = __dsub_rn(1.0, wy0);
    const double w00 = __dmul_rn(wx1, wy1), w01 = __dmul_rn(wx0, wy1);
    const double w10 = __dmul_rn(wx1, wy0), w11 = __dmul_rn(wx0, wy0);
    double r = __dmul_rn((double)p00, w00);
    r = __dadd_rn(r, __dmul_rn((double)p01, w01));
    r = __dadd_rn(r, __dmul_rn((double)p10, w10));
    r = __dadd_rn(r, __dmul_rn((double)p11, w11));
    const int v = __double2int_rn(r);
    return min(max(v, 0), 255);
}

// Exact float of a byte without a conversion instruction: 2^23 + b has b in
// its low mantissa bits.
__device__ __forceinline__ float byteToFloat(uint32_t b) { return __int_as_float(0x4B000000u | b) - 8388608.f; }

// The remap of one pixel: the texel fetch and the LUT + bilinear finish.
struct RemapTap {
    uint32_t t00, t01, t10, t11;  // texels (x0,y0) (x1,y0) (x0,y1) (x1,y1)
    float fx, fy;                 // fractional coordinates
    int x0, y0;                   // -1: the map is invalid here
};

// Integer parts use a float addition at 2^23 scale (round toward zero: the
// floor of a non-negative coordinate), which keeps the conversion unit out
// of the inner loop.
__device__ __forceinline__ void remapFetch(float2 m, const uint8_t* base, long long pitch, int fmt, int sw, int sh,
                                           RemapTap& p)
{
    p.x0 = -1;
    if (!(m.x >= 0.f && m.y >= 0.f && m.x < (float)sw && m.y < (float)sh)) return;
    const float tx = __fadd_rz(m.x, 8388608.f), ty = __fadd_rz(m.y, 8388608.f);  // 2^23 + floor
    const int x0 = __float_as_int(tx) - 0x4B000000, y0 = __float_as_int(ty) - 0x4B000000;
    const int x1 = min(x0 + 1, sw - 1), y1 = min(y0 + 1, sh - 1);
    const uint8_t* r0 = base + (size_t)y0 * pitch;
    const uint8_t* r1 = base + (size_t)y1 * pitch;
    const long long bytes = pitch * sh;
    p.t00 = loadTexel(r0, x0, fmt, base, bytes);
    p.t01 = loadTexel(r0, x1, fmt, base, bytes);
    p.t10 = loadTexel(r1, x0, fmt, base, bytes);
    p.t11 = loadTexel(r1, x1, fmt, base, bytes);
    p.fx = m.x - (tx - 8388608.f);  // exact
    p.fy = m.y - (ty - 8388608.f);
    p.x0 = x0;
    p.y0 = y0;
}

// Returns B | G << 8 | R << 16 (0 where the map is invalid).
// The fp32 result of a pixel's three channels.  Where a channel lies within
// 2e-4 of a rounding tie, fp32 cannot decide the byte: with exact, that
// channel is recomputed with the reference's double sequence; without,
// nearTie is set and the caller has the pixel recomputed (k_remap_fix).
template <bool kExact>
__device__ __forceinline__ uint32_t remapFinish(const RemapTap& p, float2 m, const uint8_t* lut, bool& nearTie)
{
    if (p.x0 < 0) return 0;
    const float gx = 1.f - p.fx, gy = 1.f - p.fy;
    const float w00 = gx * gy, w01 = p.fx * gy, w10 = gx * p.fy, w11 = p.fx * p.fy;
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const uint32_t sel = 0x4440u | (uint32_t)c;  // byte c, zero-extended
        const int p00 = lut[c * 256 + __byte_perm(p.t00, 0, sel)];
        const int p01 = lut[c * 256 + __byte_perm(p.t01, 0, sel)];
        const int p10 = lut[c * 256 + __byte_perm(p.t10, 0, sel)];
        const int p11 = lut[c * 256 + __byte_perm(p.t11, 0, sel)];
        const float r = fmaf(byteToFloat(p11), w11,
                             fmaf(byteToFloat(p10), w10, fmaf(byteToFloat(p01), w01, byteToFloat(p00) * w00)));
        // r lies in [-1e-4, 255 + 1e-4]; 1.5 * 2^23 + r rounds r to the
        // nearest integer, ties to even, in the low mantissa bits
        const float t = r + 12582912.f;
        int v = __float_as_int(t) - 0x4B400000;
        const bool tie = fabsf(r - (t - 12582912.f)) > 0.4998f;  // within 2e-4 of a tie
        if (kExact) {
            if (tie) v = bilinearExact((double)m.x, (double)m.y, p.x0, p.y0, p00, p01, p10, p11);
        } else {
            nearTie |= tie;
        }
        out |= (uint32_t)v << (8 * c);
    }
    return out;
}

// Map-free remap: the source coordinate of canvas pixel (cx, cy) in fp32,
// the steps of Remap::remapImage (source/Warp/Remap.cpp:356-514) as the
// reference's dstToSrc takes them (source/CudaAccel/CudaReproject.cu:81-264),
// which keeps them in double.  Within about 1e-3 px of the FP64 maps; the
// caller clamps the result into the frame, coverage comes from the FP64
// geometry of prepare.
__device__ __forceinline__ float2 remapPointF(const RemapParamF& m, float cx, float cy)
{
    constexpr float kPiF = 3.14159265358979323846f;
    const float xs = cx - (m.srcTX - 0.5f), ys = cy - (m.srcTY - 0.5f);
    float xd = xs + m.rot1;
    while (xd < -m.rot0) xd += 2.f * m.rot0;
    while (xd > m.rot0) xd -= 2.f * m.rot0;
    float phi = xd / m.distance;
    float theta = -ys / m.distance + kPiF / 2.f;
    if (theta < 0.f) { theta = -theta; phi += kPiF; }
    if (theta > kPiF) { theta = kPiF - (theta - kPiF); phi += kPiF; }
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    const float u0 = st * sp, u1 = ct, u2 = st * cp;
    const float v0 = m.mt[0] * u0 + m.mt[3] * u1 + m.mt[6] * u2;
    const float v1 = m.mt[1] * u0 + m.mt[4] * u1 + m.mt[7] * u2;
    const float v2 = m.mt[2] * u0 + m.mt[5] * u1 + m.mt[8] * u2;
    const float r = sqrtf(v0 * v0 + v1 * v1);
    const float th0 = r == 0.f ? 0.f : m.distance * atan2f(r, v2) / r;
    float x = th0 * v0, y = th0 * v1;
    if (m.type == 0) {
        const float rr = sqrtf(x * x + y * y);
        const float th = rr / m.distance;
        const float rho = th >= kPiF / 2.f ? 1.6e16f : (th == 0.f ? 1.f : tanf(th) / th);
        x *= rho;
        y *= rho;
    }
    x *= m.scale0;
    y *= m.scale1;
    const float rt = sqrtf(x * x + y * y) / m.rad[4];
    const float sc = rt < m.rad[5] ? ((m.rad[3] * rt + m.rad[2]) * rt + m.rad[1]) * rt + m.rad[0] : 1000.f;
    x *= sc;
    y *= sc;
    y += m.vertical;
    x += m.horizontal;
    const float xo = x + m.shear0 * y, yo = y + m.shear1 * x;
    return make_float2(xo + (m.destTX - 0.5f), yo + (m.destTY - 0.5f));
}

// The map value of a map-free pixel: -1 where the camera does not cover it,
// else the fp32 coordinate clamped into the frame.
__device__ __forceinline__ float2 mapFreeValue(const RemapParamF& m, uint32_t covWord, int lx, int cx, int cy, int sw,
                                               int sh)
{
    if (!((covWord >> lx) & 1u)) return make_float2(-1.f, -1.f);
    const float2 v = remapPointF(m, (float)cx, (float)cy);
    return make_float2(fminf(fmaxf(v.x, 0.f), __int_as_float(__float_as_int((float)sw) - 1)),
                       fminf(fmaxf(v.y, 0.f), __int_as_float(__float_as_int((float)sh) - 1)));
}

// The remap of one pixel, exact (kExact) or fp32 with the near-tie flag.
template <bool kExact = true>
__device__ __forceinline__ uint32_t remapPixel(float2 m, const uint8_t* base, long long pitch, int fmt, int sw,
                                               int sh, const uint8_t* lut, bool& nearTie)
{
    RemapTap p;
    remapFetch(m, base, pitch, fmt, sw, sh, p);
    return remapFinish<kExact>(p, m, lut, nearTie);
}

__device__ __forceinline__ uint32_t remapPixel(float2 m, const uint8_t* base, long long pitch, int fmt, int sw,
                                               int sh, const uint8_t* lut)
{
    bool unused = false;
    return remapPixel<true>(m, base, pitch, fmt, sw, sh, lut, unused);
}

// Level-0 remap over the covered 32x16 tiles of every camera; each thread
// remaps two pixels (rows ly and ly + 8) so two independent gathers are in
// flight; the tile's map is 512 consecutive float2.  A CTA walks a
// contiguous run of items (camera-major, so the camera rarely changes): the
// camera's constants and LUT are reloaded only when it does, and the next
// item's map is loaded before the current item's gathers.
struct RemapSeg {
    const RemapItem* items;
    int prefix, end;
    const RigDev* R;
    const FrameDev* F;
};

__device__ __forceinline__ RemapSeg remapSeg(const Segment* segs, int nsegs, int s, int total)
{
    const Segment& sg = segs[s];
    return {static_cast<const RemapItem*>(sg.items), sg.prefix, s + 1 < nsegs ? segs[s + 1].prefix : total, sg.rig,
            sg.frame};
}

// Items are handed out in chunks of kRemapChunk through `counter` (zero at
// launch); the next chunk is fetched one chunk ahead, so the next item and
// its map are always known before the current item is gathered.
constexpr int kRemapChunk = 8;

// The map value of pixel (lx, row) of a remap tile: from the resident maps,
// or, map-free, from the coverage bits (the FP64 coverage of prepare) and the
// fp32 geometry.
__device__ __forceinline__ float2 remapMapValue(const RigDev& R, const RemapItem& itm, int lx, int row)
{
    const long long tiles = R.numRemapItems;
    if (R.maps) {
        const float2* mt = R.maps + (size_t)itm.mapTile * (kRemapTW * kRemapTH) + row * kRemapTW + lx;
        return ldChecked(mt, R.maps, tiles * kRemapTW * kRemapTH * (long long)sizeof(float2));
    }
    const uint32_t* cw = R.covTiles + (size_t)itm.mapTile * kRemapTH;
    const uint32_t bits = ldChecked(cw + row, R.covTiles, tiles * kRemapTH * 4);
    return mapFreeValue(R.camsF[itm.cam], bits, lx, itm.tx * kRemapTW + lx, itm.ty * kRemapTH + row, R.srcW,
                        R.srcH);
}

// The exact pixel: the reference's double sequence where fp32 lies near a
// tie; the camera's LUT is read from global memory.
__device__ __forceinline__ void remapFixPixel(const FrameDev& F, const RigDev& R, float2 m, uint32_t pixel, int cam)
{
    const uint32_t pitch = (uint32_t)R.lv[0].pitch;
    if (pixel % pitch >= (uint32_t)R.W || pixel / pitch >= (uint32_t)R.H) return;  // a tile's part off the canvas
    const uint32_t v = remapPixel(m, F.src[cam], F.srcPitch[cam], F.srcFmt, R.srcW, R.srcH, F.luts + cam * 768);
    uint32_t* g = reinterpret_cast<uint32_t*>(R.lv[0].G) + (size_t)cam * R.lv[0].camStride + pixel;
    if (inside(g, R.lv[0].G, gBytes(R, R.lv[0]))) *g = v;
}

// The rare pixels whose fp32 remap lies near a rounding tie (about 0.1% of
// them) get the reference's double sequence.  Inline (kDefer false), the
// check with its out-of-line double call costs every pixel (a quarter of the
// kernel's instructions; keeping the double sequence inline spills).
// Deferred, a warp appends such pixels to the launch's list (tieCount, ties:
// room for tieCap entries, one atomic per warp) and k_remap_fix recomputes
// them before anything reads level 0: the remap is faster, and the short
// extra launch costs latency only when nothing else is in flight.  kFmt
// fixes the sources' format at compile time (PS_FMT_BGR32, the common
// case, saves the per-texel format test) or leaves it to the frame (0).
template <bool kDefer, int kFmt>
__global__ void __launch_bounds__(kThreads, 4) k_remap(const Segment* __restrict__ segs, int nsegs, int total,
                                                       int* __restrict__ counter, int* __restrict__ tieCount,
                                                       RemapTie* __restrict__ ties, int tieCap)
{
    __shared__ uint8_t lut[3 * 256];
    __shared__ int s_grab;
    auto grab = [&] {  // all threads together
        __syncthreads();
        if (threadIdx.x == 0) s_grab = atomicAdd(counter, kRemapChunk);
        __syncthreads();
        return s_grab;
    };
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    // The hand-out counter, items, descriptors and maps are written before
    // the launch sequence, not by a kernel: the first chunk and its map are
    // fetched while the previous kernel finishes.
    int it = grab(), end = 0, nextBegin = total, s = 0;
    RemapSeg cur{};
    RemapItem item{};
    float2 m0{}, m1{};
    if (it < total) {
        end = min(it + kRemapChunk, total);
        nextBegin = grab();
        s = findSegment(segs, nsegs, it, 0);
        cur = remapSeg(segs, nsegs, s, total);
        item = cur.items[it - cur.prefix];
        m0 = remapMapValue(*cur.R, item, lx, ly);
        m1 = remapMapValue(*cur.R, item, lx, ly + 8);
    }
    waitPrevGrid();
    allowNextGrid();
    if (it >= total) return;
    // constants of the loaded camera
    int camSeg = -1, cam = -1;
    const FrameDev* camF = nullptr;  // the frame and rig of the loaded camera
    const RigDev* camR = nullptr;
    const uint8_t* base = nullptr;
    long long pitch = 0;
    int fmt = 0, sw = 0, sh = 0, W = 0, H = 0, gpitch = 0;
    uint32_t* G = nullptr;
    const void* gLo = nullptr;  // the level-0 buffer of the camera's rig and its extent (checked build)
    long long gExt = 0;
    for (;;) {
        if (item.cam != cam || s != camSeg) {  // uniform across the block
            const FrameDev& F = *cur.F;
            const RigDev& R = *cur.R;
            cam = item.cam;
            camSeg = s;
            camF = &F;
            camR = &R;
            base = F.src[cam];
            pitch = F.srcPitch[cam];
            fmt = F.srcFmt;
            sw = R.srcW;
            sh = R.srcH;
            W = R.W;
            H = R.H;
            gpitch = R.lv[0].pitch;
            G = reinterpret_cast<uint32_t*>(R.lv[0].G) + (size_t)cam * R.lv[0].camStride;
            gLo = R.lv[0].G;
            gExt = gBytes(R, R.lv[0]);
            __syncthreads();
            const uint8_t* src = F.luts + cam * 768;
            for (int k = threadIdx.x; k < 768; k += kThreads) lut[k] = __ldg(src + k);
            __syncthreads();
        }
        // the next item (the rest of this chunk, else the next chunk's first) and its map
        const int nit = it + 1 < end ? it + 1 : (nextBegin < total ? nextBegin : -1);
        RemapItem nitem = item;
        float2 n0 = m0, n1 = m1;
        if (nit >= 0) {
            if (nit >= cur.end) {
                s = findSegment(segs, nsegs, nit, s);
                cur = remapSeg(segs, nsegs, s, total);
            }
            nitem = cur.items[nit - cur.prefix];
            n0 = remapMapValue(*cur.R, nitem, lx, ly);
            n1 = remapMapValue(*cur.R, nitem, lx, ly + 8);
        }
        bool tie0 = false, tie1 = false;
        const uint32_t v0 = remapPixel<!kDefer>(m0, base, pitch, kFmt ? kFmt : fmt, sw, sh, lut, tie0);
        const uint32_t v1 = remapPixel<!kDefer>(m1, base, pitch, kFmt ? kFmt : fmt, sw, sh, lut, tie1);
        const int x = item.tx * kRemapTW + lx, y0 = item.ty * kRemapTH + ly, y1 = y0 + 8;
        if (kDefer) {
            const uint32_t b0 = __ballot_sync(0xffffffffu, tie0), b1 = __ballot_sync(0xffffffffu, tie1);
            if (b0 | b1) {  // the warp's near-tie pixels, one atomic for the warp
                int e = 0;
                if (lx == 0) e = atomicAdd(tieCount, __popc(b0) + __popc(b1));
                e = __shfl_sync(0xffffffffu, e, 0);
                const uint32_t below = (1u << lx) - 1u;
                const int e0 = e + __popc(b0 & below), e1 = e + __popc(b0) + __popc(b1 & below);
                if (tie0 && e0 < tieCap) ties[e0] = {camF, camR, m0.x, m0.y, (uint32_t)((size_t)y0 * gpitch + x), cam};
                if (tie1 && e1 < tieCap) ties[e1] = {camF, camR, m1.x, m1.y, (uint32_t)((size_t)y1 * gpitch + x), cam};
            }
        }
        if (x < W) {
            if (y0 < H && inside(G + (size_t)y0 * gpitch + x, gLo, gExt)) G[(size_t)y0 * gpitch + x] = v0;
            if (y1 < H && inside(G + (size_t)y1 * gpitch + x, gLo, gExt)) G[(size_t)y1 * gpitch + x] = v1;
        }
        if (nit < 0) break;
        if (it + 1 >= end) {  // into the next chunk; fetch the one after it
            end = min(nextBegin + kRemapChunk, total);
            nextBegin = grab();
        }
        it = nit;
        item = nitem;
        m0 = n0;
        m1 = n1;
    }
}

// The exact recompute of the pixels k_remap put on the launch's list
// (ties[0 .. *tieCount)), one thread per entry.  An entry carries its frame,
// rig, map value and pixel, so the recompute is a short chain of loads.
// Most frames list none.  A list that overflowed (more than tieCap entries)
// has every pixel of the launch recomputed, tile by tile.
__global__ void __launch_bounds__(kThreads) k_remap_fix(const Segment* __restrict__ segs, int nsegs, int total,
                                                        const int* __restrict__ tieCount,
                                                        const RemapTie* __restrict__ ties, int tieCap)
{
    waitPrevGrid();
    allowNextGrid();
    const int listed = __ldcg(tieCount);
    const long long stride = (long long)gridDim.x * kThreads;
    const long long first = blockIdx.x * (long long)kThreads + threadIdx.x;
    if (listed <= tieCap) {
        for (long long e = first; e < listed; e += stride) {
            const RemapTie t = ties[e];
            remapFixPixel(*t.frame, *t.rig, make_float2(t.mx, t.my), t.pixel, t.cam);
        }
        return;
    }
    for (long long e = first; e < (long long)total * kThreads * 2; e += stride) {  // the list overflowed
        const int it = (int)(e / (kThreads * 2)), t = (int)(e % (kThreads * 2)) >> 1, half = (int)(e & 1);
        const int s = findSegment(segs, nsegs, it, 0);
        const RemapSeg cur = remapSeg(segs, nsegs, s, total);
        const RemapItem item = cur.items[it - cur.prefix];
        const int lx = t & 31, row = (t >> 5) + half * 8;
        const int x = item.tx * kRemapTW + lx, y = item.ty * kRemapTH + row;
        if (x < cur.R->W && y < cur.R->H)
            remapFixPixel(*cur.F, *cur.R, remapMapValue(*cur.R, item, lx, row),
                          (uint32_t)((size_t)y * cur.R->lv[0].pitch + x), item.cam);
    }
}

// ============================================================================
// k_linear: the linear-blend render (highQualityBlend == 0, CudaPanoramaRender2::
// render, source/Task/RicohUtil.cpp:1269-1286): per canvas pixel
//   accum = sum over cameras, in index order, of remap_i * w_i
// in fp32 with one rounded product and one rounded sum per camera
// (reprojectWeightedAccumulateTo32F, source/Warp/ZReproject.cpp:606-633),
// then convertTo(CV_8U): round half to even, saturate.  One 32x16 canvas
// tile per item (all tiles are items, so uncovered tiles are written 0);
// each thread two pixels (rows ly and ly + 8).  The LUTs of all cameras of
// the current rig are staged in shared memory.
// ============================================================================
__device__ __forceinline__ void storeBgr(const FrameDev& F, int x, int y, int H, uint32_t v)
{
    uint8_t* row = F.out + (size_t)y * F.outPitch;
    if (!insideRange(row + (F.outFmt == PS_FMT_BGR32 ? 4 : 3) * x, F.outFmt == PS_FMT_BGR32 ? 4 : 3, F.out,
                     F.outPitch * H))
        return;
    if (F.outFmt == PS_FMT_BGR32) {
        reinterpret_cast<uint32_t*>(row)[x] = v;
    } else {
        row[3 * x] = v & 0xFF;
        row[3 * x + 1] = (v >> 8) & 0xFF;
        row[3 * x + 2] = (v >> 16) & 0xFF;
    }
}

__device__ __forceinline__ uint32_t roundSaturate3(const float* a)
{
    uint32_t v = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) v |= (uint32_t)min(max(__float2int_rn(a[c]), 0), 255) << (8 * c);
    return v;
}

__global__ void __launch_bounds__(kThreads) k_linear(const Segment* __restrict__ segs, int nsegs, int total)
{
    extern __shared__ uint8_t luts[];  // 768 bytes per camera of the current rig
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    int s = 0, loaded = -1;
    waitPrevGrid();
    allowNextGrid();
    for (int it = blockIdx.x; it < total; it += gridDim.x) {  // uniform across the CTA
        s = findSegment(segs, nsegs, it, s);
        const Segment& sg = segs[s];
        const RigDev& R = *sg.rig;
        const FrameDev& F = *sg.frame;
        if (s != loaded) {
            __syncthreads();
            for (int k = threadIdx.x; k < R.n * 768; k += kThreads) luts[k] = __ldg(F.luts + k);
            __syncthreads();
            loaded = s;
        }
        const LinearItem item = static_cast<const LinearItem*>(sg.items)[it - sg.prefix];
        float a0[3] = {0.f, 0.f, 0.f}, a1[3] = {0.f, 0.f, 0.f};
        for (uint32_t q = 0; q < item.count; q++) {
            const RemapItem ri = R.remapItems[item.first + q];
            const size_t base = (size_t)ri.mapTile * (kRemapTW * kRemapTH) + threadIdx.x;
            const long long tilePx = (long long)R.numRemapItems * kRemapTW * kRemapTH;
            const float2 m0 = ldChecked(R.maps + base, R.maps, tilePx * 8);
            const float2 m1 = ldChecked(R.maps + base + kThreads, R.maps, tilePx * 8);
            const float w0 = ldChecked(R.linWeights + base, R.linWeights, tilePx * 4);
            const float w1 = ldChecked(R.linWeights + base + kThreads, R.linWeights, tilePx * 4);
            const uint8_t* src = F.src[ri.cam];
            const long long pitch = F.srcPitch[ri.cam];
            const uint8_t* lut = luts + ri.cam * 768;
            const uint32_t v0 = remapPixel(m0, src, pitch, F.srcFmt, R.srcW, R.srcH, lut);
            const uint32_t v1 = remapPixel(m1, src, pitch, F.srcFmt, R.srcW, R.srcH, lut);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                a0[c] = __fadd_rn(a0[c], __fmul_rn(byteToFloat((v0 >> (8 * c)) & 0xFF), w0));
                a1[c] = __fadd_rn(a1[c], __fmul_rn(byteToFloat((v1 >> (8 * c)) & 0xFF), w1));
            }
        }
        const int x = item.tx * kRemapTW + lx, y0 = item.ty * kRemapTH + ly, y1 = y0 + 8;
        if (x < R.W) {
            if (y0 < R.H) storeBgr(F, x, y0, R.H, roundSaturate3(a0));
            if (y1 < R.H) storeBgr(F, x, y1, R.H, roundSaturate3(a1));
        }
    }
}

// Standalone cudaReprojectTo16S with an optional LUT: full-canvas maps,
// int16x4 output (B, G, R, 0).
__global__ void __launch_bounds__(kThreads) k_reproject16s(const uint8_t* __restrict__ src, long long srcPitch,
                                                           int sw, int sh, int fmt, const float* __restrict__ xmap,
                                                           const float* __restrict__ ymap, long long mapPitch,
                                                           int W, int H, const uint8_t* __restrict__ glut,
                                                           short4* dst, long long dstPitch)
{
    __shared__ uint8_t lut[3 * 256];
    for (int k = threadIdx.x; k < 768; k += kThreads) lut[k] = glut ? glut[k] : (uint8_t)(k & 255);
    __syncthreads();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const float2 m = make_float2(reinterpret_cast<const float*>(reinterpret_cast<const uint8_t*>(xmap) + y * mapPitch)[x],
                                 reinterpret_cast<const float*>(reinterpret_cast<const uint8_t*>(ymap) + y * mapPitch)[x]);
    const uint32_t v = remapPixel(m, src, srcPitch, fmt, sw, sh, lut);
    reinterpret_cast<short4*>(reinterpret_cast<uint8_t*>(dst) + y * dstPitch)[x] =
        make_short4((short)(v & 0xFF), (short)((v >> 8) & 0xFF), (short)((v >> 16) & 0xFF), 0);
}

// ============================================================================
// k_pyrdown: pyrDown16SC4To16SC4 with alpha scale
// (source/CudaAccel/CudaPyramid2.cu:436-542): per output pixel
//   S = sum_{5x5} [1 4 6 4 1]^2 * G_j(2y+dy, 2x+dx), rows reflect-101,
//   columns wrap;  G_{j+1} = alpha ? (S << 8) / alpha : 0.
// With alpha = 256*m this is floor(S / m), evaluated exactly as
// (S * ceil(2^24 / m)) >> 24 (exact for S < 65793; S <= 65280 here).
// One CTA produces a 32x16 output tile of one camera from its 67x35 input
// tile.  Warp w owns output rows 2w and 2w + 1, i.e. input rows 4w .. 4w+6:
// lane l loads input columns 2l and 2l + 1 of those seven rows (lanes 0..2
// also column 64 + l), forms the vertical sums of both output rows in
// registers, two channels per 32-bit word, and hands them to the warp
// through the warp's own rows of shared memory; lane l then filters output
// columns 2(l % 16) and 2(l % 16) + 1 of output row 2w + l / 16.  No step
// waits for another warp.
// ============================================================================
constexpr int kDInW = 2 * kDownTW + 3;   // 67 input columns
constexpr int kDVP = kDInW + 1;          // 68: row stride of the vertical sums (16-byte aligned rows)
constexpr int kDWarps = kThreads / 32;   // 8
constexpr int kDRows = 7;                // input rows of a warp's two output rows
static_assert(kDownTH == 2 * kDWarps, "a warp owns two output rows");
static_assert(kDownTW == 32 && kDInW - 64 <= 32, "lanes cover the input columns as 2 x 32 + 3");

struct alignas(16) DownSmem {
    uint2 v[kDWarps][2][kDVP];  // vertical sums (B|R, G|X lanes) of each warp's two output rows
    uint32_t magic[257];
};

__device__ __forceinline__ void initMagic(uint32_t* magic)
{
    for (int m = threadIdx.x; m < 257; m += blockDim.x) magic[m] = m ? (uint32_t)((16777216u + m - 1) / m) : 0u;
}

// Loads of pyramid levels.  A level written earlier in the same launch (the
// tail kernel's levels) is read through L2 (ld.global.cg); one written by an
// earlier launch may use the read-only path.
template <bool kFresh, class T>
__device__ __forceinline__ T ldLevel(const T* p)
{
    if constexpr (kFresh) return __ldcg(p);
    else return __ldg(p);
}

// A lane's part of its warp's input rows, and the alpha divisors of the
// lane's two outputs (low half: the left one).
struct DownRegs {
    uint32_t a[kDRows], b[kDRows];  // input columns 2*lane, 2*lane + 1
    uint32_t c[kDRows];             // input column 64 + lane (lanes 0..2)
    uint32_t m;
};

__device__ __forceinline__ bool downInterior(const RigDev& R, const DownItem& item)
{
    const LevelDev& Ls = R.lv[item.level - 1];
    const int ix0 = 2 * item.tx * kDownTW - 2, iy0 = 2 * item.ty * kDownTH - 2;
    return ix0 >= 0 && iy0 >= 0 && ix0 + kDInW <= Ls.w && iy0 + 2 * kDownTH + 3 <= Ls.h;
}

// The lane's loads for a tile.  Interior tiles read whole rows (8-byte loads:
// the first input column is even and rows are 256-byte aligned); tiles whose
// input crosses the level's border map every row and column with the
// reference's reflect-101 / wrap rules.
template <bool kFresh>
__device__ __forceinline__ void downLoad(const RigDev& R, const DownItem& item, DownRegs& g)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const LevelDev& Ls = R.lv[item.level - 1];
    const LevelDev& Ld = R.lv[item.level];
    const int ox0 = item.tx * kDownTW, oy0 = item.ty * kDownTH;
    const int ix0 = 2 * ox0 - 2, iy0 = 2 * oy0 - 2 + 4 * w;  // the warp's first input row
    const uint32_t* G = reinterpret_cast<const uint32_t*>(Ls.G) + (size_t)item.cam * Ls.camStride;
    // the lane's outputs (X, Y), (X + 1, Y): X is even, so both divisors are
    // one aligned 4-byte load (X + 1 stays inside the row pitch)
    const int X = ox0 + 2 * (lane & 15), Y = oy0 + 2 * w + (lane >> 4);
    g.m = X < Ld.w && Y < Ld.h ? ldChecked(reinterpret_cast<const uint32_t*>(Ld.Am + (size_t)item.cam * Ld.camStride +
                                                                           (size_t)Y * Ld.pitch + X),
                                           Ld.Am, wBytes(R, Ld))
                               : 0u;
    const bool extra = lane < kDInW - 64;
    const long long ext = gBytes(R, Ls);
    if (downInterior(R, item)) {
        const uint32_t* row = G + (size_t)iy0 * Ls.pitch + ix0;
#pragma unroll
        for (int r = 0; r < kDRows; r++, row += Ls.pitch) {
            const uint2* q = reinterpret_cast<const uint2*>(row) + lane;
            const uint2 v = inside(q, Ls.G, ext) ? ldLevel<kFresh>(q) : make_uint2(0, 0);
            g.a[r] = v.x;
            g.b[r] = v.y;
            g.c[r] = extra && inside(row + 64 + lane, Ls.G, ext) ? ldLevel<kFresh>(row + 64 + lane) : 0u;
        }
        return;
    }
    const int c0 = colMap(ix0 + 2 * lane, Ls.w), c1 = colMap(ix0 + 2 * lane + 1, Ls.w);
    const int c2 = extra ? colMap(ix0 + 64 + lane, Ls.w) : 0;
#pragma unroll
    for (int r = 0; r < kDRows; r++) {
        const uint32_t* row = G + (size_t)rowMap(iy0 + r, Ls.h) * Ls.pitch;
        g.a[r] = inside(row + c0, Ls.G, ext) ? ldLevel<kFresh>(row + c0) : 0u;
        g.b[r] = inside(row + c1, Ls.G, ext) ? ldLevel<kFresh>(row + c1) : 0u;
        g.c[r] = extra && inside(row + c2, Ls.G, ext) ? ldLevel<kFresh>(row + c2) : 0u;
    }
}

// [1 4 6 4 1] over five 16-bit-lane words (sums of up to 16 * 4080 stay in
// the lanes).
__device__ __forceinline__ uint32_t k5(uint32_t p0, uint32_t p1, uint32_t p2, uint32_t p3, uint32_t p4)
{
    return p0 + p4 + 4 * (p1 + p3) + 6 * p2;
}

// Vertical sums of one input column: the even output row from input rows
// 0..4, the odd one from rows 2..6.
__device__ __forceinline__ void downColumn(const uint32_t* p, uint2& e, uint2& o)
{
    uint2 u[kDRows];
#pragma unroll
    for (int r = 0; r < kDRows; r++) u[r] = unpackBytes(p[r]);
    e = make_uint2(k5(u[0].x, u[1].x, u[2].x, u[3].x, u[4].x), k5(u[0].y, u[1].y, u[2].y, u[3].y, u[4].y));
    o = make_uint2(k5(u[2].x, u[3].x, u[4].x, u[5].x, u[6].x), k5(u[2].y, u[3].y, u[4].y, u[5].y, u[6].y));
}

// The lane's vertical sums into the warp's rows.
__device__ __forceinline__ void downVertical(const DownRegs& g, DownSmem& sm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint2 ea, oa, eb, ob;
    downColumn(g.a, ea, oa);
    downColumn(g.b, eb, ob);
    __syncwarp();  // the warp's reads of its previous tile are done
    *reinterpret_cast<uint4*>(&sm.v[w][0][2 * lane]) = make_uint4(ea.x, ea.y, eb.x, eb.y);
    *reinterpret_cast<uint4*>(&sm.v[w][1][2 * lane]) = make_uint4(oa.x, oa.y, ob.x, ob.y);
    if (lane < kDInW - 64) {
        uint2 ec, oc;
        downColumn(g.c, ec, oc);
        sm.v[w][0][64 + lane] = ec;
        sm.v[w][1][64 + lane] = oc;
    }
    __syncwarp();
}

// floor(S / m) of the B, G, R sums (lo = B | R << 16, hi = G | X << 16):
// floor(S / m) = floor(S * ceil(2^24 / m) / 2^24) = umulhi(S << 8, ceil(2^24 / m)).
__device__ __forceinline__ uint32_t downDivide(uint32_t lo, uint32_t hi, uint32_t m, const uint32_t* magic)
{
    if (!m) return 0;
    const uint32_t mg = magic[m];
    const uint32_t b = __umulhi((lo & 0xFFFFu) << 8, mg);
    const uint32_t r = __umulhi((lo >> 16) << 8, mg);
    const uint32_t gg = __umulhi((hi & 0xFFFFu) << 8, mg);
    return b | (gg << 8) | (r << 16);
}

// Horizontal pass of the lane's two outputs from the warp's rows, and the
// stores.  m: the divisors loaded with the tile.
__device__ __forceinline__ void downHorizontal(const RigDev& R, const DownItem& item, uint32_t m, const DownSmem& sm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int k = lane & 15, rsel = lane >> 4;
    // output columns 2k and 2k + 1 read vertical sums 4k .. 4k + 4 and 4k + 2 .. 4k + 6
    const uint2* vr = &sm.v[w][rsel][4 * k];
    const uint4 q01 = *reinterpret_cast<const uint4*>(vr);
    const uint4 q23 = *reinterpret_cast<const uint4*>(vr + 2);
    const uint4 q45 = *reinterpret_cast<const uint4*>(vr + 4);
    const uint2 q6 = vr[6];
    const uint32_t lo0 = k5(q01.x, q01.z, q23.x, q23.z, q45.x), hi0 = k5(q01.y, q01.w, q23.y, q23.w, q45.y);
    const uint32_t lo1 = k5(q23.x, q23.z, q45.x, q45.z, q6.x), hi1 = k5(q23.y, q23.w, q45.y, q45.w, q6.y);
    const uint32_t out0 = downDivide(lo0, hi0, m & 0xFFFFu, sm.magic);
    const uint32_t out1 = downDivide(lo1, hi1, m >> 16, sm.magic);
    const LevelDev& Ld = R.lv[item.level];
    const int X = item.tx * kDownTW + 2 * k, Y = item.ty * kDownTH + 2 * w + rsel;
    if (X < Ld.w && Y < Ld.h) {
        uint32_t* dst = reinterpret_cast<uint32_t*>(Ld.G) + (size_t)item.cam * Ld.camStride + (size_t)Y * Ld.pitch + X;
        const long long ext = gBytes(R, Ld);
        if (X + 1 < Ld.w) {
            if (inside(reinterpret_cast<uint2*>(dst), Ld.G, ext)) *reinterpret_cast<uint2*>(dst) = make_uint2(out0, out1);
        } else if (inside(dst, Ld.G, ext)) {
            dst[0] = out0;
        }
    }
}

// One 32x16 output tile of one camera (all warps of the CTA; the magic table
// is ready), without overlap (the tail kernel's few tiles).
template <bool kFresh>
__device__ __forceinline__ void pyrDownTile(const RigDev& R, const DownItem item, DownSmem& sm)
{
    DownRegs g;
    downLoad<kFresh>(R, item, g);
    downVertical(g, sm);
    downHorizontal(R, item, g.m, sm);
}

// One CTA walks a contiguous run of tiles; the next tile's loads are issued
// before the current tile's horizontal pass, so their latency overlaps it.
__global__ void __launch_bounds__(kThreads, 5) k_pyrdown(const Segment* __restrict__ segs, int nsegs, int total)
{
    __shared__ DownSmem sm;
    initMagic(sm.magic);
    int s = 0, begin, end;
    itemRange(total, begin, end);
    // Items and descriptors are written before the launch sequence, not by
    // a kernel: the first tile's are read while the previous kernel finishes.
    const RigDev* R = nullptr;
    DownItem item{};
    if (begin < end) {
        s = findSegment(segs, nsegs, begin, s);
        R = segs[s].rig;
        item = static_cast<const DownItem*>(segs[s].items)[begin - segs[s].prefix];
    }
    waitPrevGrid();
    allowNextGrid();
    if (begin >= end) return;
    __syncthreads();  // the magic table
    DownRegs g;
    downLoad<false>(*R, item, g);
    for (int it = begin; it < end; it++) {
        const bool more = it + 1 < end;
        int sn = s;
        DownItem next = item;
        if (more) {
            sn = findSegment(segs, nsegs, it + 1, s);
            next = static_cast<const DownItem*>(segs[sn].items)[it + 1 - segs[sn].prefix];
        }
        downVertical(g, sm);
        const uint32_t m = g.m;
        if (more) downLoad<false>(*segs[sn].rig, next, g);
        downHorizontal(*R, item, m, sm);
        s = sn;
        R = segs[s].rig;
        item = next;
    }
}

// ============================================================================
// k_blend: one canvas level of the blend, all cameras at once.
//   For each camera i whose weight touches the tile:
//     U = pyrUp(G_{i,j+1})            pyrUp16SC4To16SC4, CudaPyramid2.cu:628-710
//     L = G_{i,j} - U  (L_L = G_L)    subtract16SC4, :836-845
//     R += w_ij * L, W += w_ij        accumulate16SC4To32SC4, :759-773
//   N = full ? (R + 128) >> 8 : R / max(W, 1)     normalize32SC4, :749-791
//   C_j = N + pyrUp32(C_{j+1})        restoreImageFromLaplacePyramid,
//                                     CudaMultibandBlend.cpp:220-231
//   level 0: out = clamp(C_0, 0, 255), 0 where no camera covers
//   (convertTo(CV_8U) + setTo(0, maskNot), CudaMultibandBlend.cpp:820-822).
// A tile whose only camera has weight 256 on every pixel has N = L exactly
// (R = 256 L, W = 256; (256 L + 128) >> 8 = L), so it skips the weights.
//
// A tile is 64x16 canvas pixels; consumer thread t (of 256) owns the 2x2
// block at (2*(t%32), 2*(t/32)), so the zero-inserted upsample's three
// footprint rows serve both of its rows and the YUV chroma of the block is
// its own.  Work flows through a 2-stage shared-memory ring of "units" (a
// tile and up to two of its cameras).  A
// dedicated producer warp stages each unit with bulk asynchronous copies of
// whole rows -- the cameras' G_j and weight rows, their G_{j+1} footprint
// rows and, with a tile's last unit, the C_{j+1} footprint rows -- completing
// on the stage's "full" mbarrier; the eight consumer warps compute from
// shared memory and release the stage on its "empty" mbarrier.  Tiles whose
// footprints cross the canvas border (horizontal wrap, vertical
// reflect-101) are staged by the consumers with the reference's index
// mapping.
// ============================================================================
constexpr int kFW = kBlendTW / 2 + 2;  // 34: footprint columns fx0 .. fx0+33
constexpr int kFH = kBlendTH / 2 + 2;  // 10: footprint rows    fy0 .. fy0+9
constexpr int kBStages = 2;
constexpr int kCamsPerUnit = 2;
constexpr int kFpW = 40;   // staged footprint row: columns fx0-3 .. fx0+36 (16-byte aligned start)
constexpr int kCfW = 36;   // staged collapse footprint row: columns fx0-1 .. fx0+34
constexpr int kMaxSmemSegs = 64;
constexpr int kConsumers = kThreads;          // 8 warps
constexpr int kBlendThreads = kConsumers + 32;  // + the producer warp

// One unit's shared-memory stage: NC cameras of one tile (k_blend stages
// two cameras per unit in a ring; the tail kernel stages up to eight at once).
// Every camera's part starts on a 128-byte boundary, as the bulk tensor
// copies into it require: the footprint of a camera is kFH rows of kFpW
// words (a dense box), padded to kFpCam words.
template <int NC>
struct alignas(128) BlendStageT {
    static constexpr int kCams = NC;
    static constexpr int kFpCam = (kFH * kFpW + 31) / 32 * 32;
    uint32_t gj[NC][kBlendTH][kBlendTW];  // G_j, uchar4
    uint16_t w[NC][kBlendTH][kBlendTW];   // weights
    uint32_t fpw[NC][kFpCam];             // G_{j+1} footprint: row r, column c at [r * kFpW + c]
    uint2 cf[kFH][kCfW];                  // C_{j+1} footprint (short4 bits)
};
using BlendStage = BlendStageT<kCamsPerUnit>;
static_assert(offsetof(BlendStage, w) % 128 == 0 && offsetof(BlendStage, fpw) % 128 == 0 &&
                  offsetof(BlendStage, cf) % 128 == 0 && sizeof(BlendStage::gj[0]) % 128 == 0 &&
                  sizeof(BlendStage::w[0]) % 128 == 0 && sizeof(BlendStage::fpw[0]) % 128 == 0,
              "every bulk tensor copy destination starts on a 128-byte boundary");
constexpr int kTailCamsPerUnit = 8;

// What the consumers need of a unit besides its stage: the level geometry
// and the frame's output, resolved once per unit (in k_blend by the
// producer warp, so the consumers read it from shared memory).
struct UnitGeo {
    int w, h, pitch, full, hasUp, outFmt;
    short4* C;              // collapsed result of the unit's level (j >= 1)
    const uint8_t* um;      // union mask (level 0, partially covered tiles)
    uint8_t* out;           // BGR canvas or Y plane
    uint8_t* outU;          // U (YUV420P) or UV (NV12) plane
    uint8_t* outV;          // V plane (YUV420P)
    long long outPitch, outCPitch, outVPitch;
};

__device__ __forceinline__ void fillGeo(UnitGeo& g, const RigDev& R, const FrameDev& F, int j)
{
    const LevelDev& Lj = R.lv[j];
    g.w = Lj.w;
    g.h = Lj.h;
    g.pitch = Lj.pitch;
    g.full = R.full;
    g.hasUp = j < R.L;
    g.outFmt = F.outFmt;
    g.C = Lj.C;
    g.um = R.unionMask;
    g.out = F.out;
    g.outU = F.outU;
    g.outV = F.outV;
    g.outPitch = F.outPitch;
    g.outCPitch = F.outCPitch;
    g.outVPitch = F.outVPitch;
}

struct UnitInfo {
    uint4 raw;
    int seg, chunk, valid, staged;  // staged: copies issued by the producer
    UnitGeo geo;
};

// ---- BT.601 studio-range conversion (cvtBGRToYUV2x2Block,
// ImageProc.cu:44-95): 20-bit fixed point, Y = 16 + ..., chroma = 128 + ...
// These are the standard BT.601 coefficients scaled by 2^20; the chroma of
// a 2x2 block is the mean of its left column's two pixels.
constexpr int kYR = 269484, kYG = 528482, kYB = 102760;
constexpr int kUR = -155188, kUG = -305135, kUB = 460324;
constexpr int kVR = 460324, kVG = -385875, kVB = -74448;
constexpr int kYuvShift = 20;
constexpr int kYuvHalf = 1 << (kYuvShift - 1);
constexpr int kYOff = (16 << kYuvShift) + kYuvHalf;
constexpr int kCOff = (128 << kYuvShift) + kYuvHalf;

__device__ __forceinline__ int clamp255(int v) { return min(max(v, 0), 255); }

// B | G << 8 | R << 16 with each channel saturated to 0..255: two
// cvt.pack.sat.u8.s32.b32 (PTX: d = sat(b) | sat(a) << 8 | c[15:0] << 16)
// instead of six min / max and the shifts.
__device__ __forceinline__ uint32_t packSatBgr(int b, int g, int r)
{
    uint32_t hi, out;
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(hi) : "r"(0), "r"(r), "r"(0));
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(out) : "r"(g), "r"(b), "r"(hi));
    return out;
}

// Luma before saturation; yuvLuma saturates it.
__device__ __forceinline__ int yuvLumaRaw(uint32_t bgr)
{
    const int b = bgr & 0xFF, g = (bgr >> 8) & 0xFF, r = (bgr >> 16) & 0xFF;
    return (kYR * r + kYG * g + kYB * b + kYOff) >> kYuvShift;
}

__device__ __forceinline__ uint32_t yuvLuma(uint32_t bgr) { return (uint32_t)clamp255(yuvLumaRaw(bgr)); }

// sat(lo) | sat(hi) << 8, each saturated to 0..255 (one cvt.pack.sat)
__device__ __forceinline__ uint32_t packSat2(int lo, int hi)
{
    uint32_t out;
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(out) : "r"(hi), "r"(lo), "r"(0));
    return out;
}

// Unshifted chroma sums of one pixel (both are non-negative).
__device__ __forceinline__ int2 yuvChromaSums(uint32_t bgr)
{
    const int b = bgr & 0xFF, g = (bgr >> 8) & 0xFF, r = (bgr >> 16) & 0xFF;
    return make_int2(kUR * r + kUG * g + kUB * b + kCOff, kVR * r + kVG * g + kVB * b + kCOff);
}

// Level-0 store of a consumer thread's 2x2 block as four Y samples and the
// block's U and V (from its left column, as cvtBGRToYUV2x2Block computes
// them).  o[0] o[1] are the top pixels, o[2] o[3] the bottom ones.
__device__ __forceinline__ void storeYuv(const UnitGeo& G, int x, int y, const uint32_t* o)
{
#pragma unroll
    for (int r = 0; r < 2; r++) {
        uint8_t* yrow = G.out + (size_t)(y + r) * G.outPitch + x;
        const uint32_t yy = packSat2(yuvLumaRaw(o[2 * r]), yuvLumaRaw(o[2 * r + 1]));
        if (!insideRange(yrow, 2, G.out, G.outPitch * G.h)) continue;
        if ((reinterpret_cast<uintptr_t>(yrow) & 1) == 0) {
            *reinterpret_cast<uint16_t*>(yrow) = (uint16_t)yy;
        } else {
            yrow[0] = (uint8_t)yy;
            yrow[1] = (uint8_t)(yy >> 8);
        }
    }
    const int2 c = yuvChromaSums(o[0]), d = yuvChromaSums(o[2]);
    const uint32_t uv = packSat2((c.x + d.x) >> (kYuvShift + 1), (c.y + d.y) >> (kYuvShift + 1));
    const uint8_t u = (uint8_t)uv, v = (uint8_t)(uv >> 8);
    const size_t cy = (size_t)(y >> 1);
    const long long cext = G.outCPitch * (G.h / 2);
    if (G.outFmt == PS_FMT_NV12) {
        uint8_t* p = G.outU + cy * G.outCPitch + x;
        if (!insideRange(p, 2, G.outU, cext)) return;
        if ((reinterpret_cast<uintptr_t>(p) & 1) == 0) {
            *reinterpret_cast<uint16_t*>(p) = (uint16_t)uv;
        } else {
            p[0] = u;
            p[1] = v;
        }
    } else {
        if (inside(G.outU + cy * G.outCPitch + (x >> 1), G.outU, cext)) G.outU[cy * G.outCPitch + (x >> 1)] = u;
        if (inside(G.outV + cy * G.outVPitch + (x >> 1), G.outV, G.outVPitch * (G.h / 2)))
            G.outV[cy * G.outVPitch + (x >> 1)] = v;
    }
}

// q-th camera of a blend tile (raw 16-byte descriptor)
__device__ __forceinline__ int tileCam(const uint4& raw, const uint8_t* camLists, int q)
{
    if (((raw.x >> 16) & 0xFF) > kInlineCams) return __ldg(camLists + raw.z + q);
    const uint32_t w = q < 4 ? raw.z : raw.w;
    return (int)((w >> (8 * (q & 3))) & 0xFF);
}

template <int NC = kCamsPerUnit>
__device__ __forceinline__ int unitChunks(const uint4& raw)
{
    const int cnt = (raw.x >> 16) & 0xFF;
    return cnt <= NC ? 1 : (cnt + NC - 1) / NC;
}

// Accumulators of a thread's 2x2 block: pixel p = 2 * row + column.
struct BlendAcc {
    int r[4][3];
    int wsum[4];
};

// Stage one unit with index-mapped loads (border tiles; every tile of the
// tail kernel).  Threads 0..kConsumers-1; the caller synchronises.
// fRow / fCol: footprint index tables (kFH / kFW ints) filled here; sync is
// the barrier over the calling threads.
// half >= 0 stages only what computeUnitRows reads for that 64x8 half:
// its eight rows and footprint rows 4*half .. 4*half+5.
template <bool kFresh, class Stage, class Sync>
__device__ __forceinline__ void stageUnitDirect(Stage& S, const RigDev& R, const uint4& raw, int chunk, int* fRow,
                                                int* fCol, Sync sync, int half = -1)
{
    const int lx = (threadIdx.x & 31) * 2;
    const int ly = half < 0 ? (threadIdx.x >> 5) * 2 : 8 * half + (threadIdx.x >> 5);
    const int rowsPerThread = half < 0 ? 2 : 1;
    const int j = raw.x & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
    const int tx = raw.y & 0xFFFF, ty = raw.y >> 16;
    const LevelDev& Lj = R.lv[j];
    const bool hasUp = j < R.L;
    const LevelDev& Lu = R.lv[hasUp ? j + 1 : j];
    const int x = tx * kBlendTW + lx, y = ty * kBlendTH + ly;
    constexpr int NC = Stage::kCams;
    const int c0 = chunk * NC;
    const int nc = max(0, min(NC, camCnt - c0));
    const bool last = chunk == unitChunks<NC>(raw) - 1;
    const int fx0 = tx * (kBlendTW / 2) - 1, fy0 = ty * (kBlendTH / 2) - 1;
    for (int q = 0; q < nc; q++) {
        const int cam = tileCam(raw, R.camLists, c0 + q);
        for (int r = 0; r < rowsPerThread; r++) {
            uint2 g = make_uint2(0, 0);
            uint32_t w = 0;
            if (y + r < Lj.h) {  // columns up to the pitch are allocated (and zero beyond the width)
                const size_t o = (size_t)cam * Lj.camStride + (size_t)(y + r) * Lj.pitch + x;
                const uint2* gp = reinterpret_cast<const uint2*>(Lj.G + o);
                const uint32_t* wp = reinterpret_cast<const uint32_t*>(Lj.Wt + o);
                if (inside(gp, Lj.G, gBytes(R, Lj))) g = ldLevel<kFresh>(gp);
                if (inside(wp, Lj.Wt, wBytes(R, Lj))) w = __ldg(wp);
            }
            *reinterpret_cast<uint2*>(&S.gj[q][ly + r][lx]) = g;
            *reinterpret_cast<uint32_t*>(&S.w[q][ly + r][lx]) = w;
        }
    }
    if (hasUp) {
        if (threadIdx.x < kFH) fRow[threadIdx.x] = rowMap(fy0 + (int)threadIdx.x, Lu.h);
        else if (threadIdx.x < kFH + kFW) fCol[threadIdx.x - kFH] = colMap(fx0 + (int)threadIdx.x - kFH, Lu.w);
        sync();
        const int rb = half < 0 ? 0 : 4 * half, nr = half < 0 ? kFH : 6;
        const int elems = nr * kFW;
        for (int k = threadIdx.x; k < nc * elems; k += kConsumers) {
            const int q = k / elems, e = k - q * elems;
            const int r = rb + e / kFW, c = e % kFW;
            const int cam = tileCam(raw, R.camLists, c0 + q);
            const uint32_t* gp = reinterpret_cast<const uint32_t*>(Lu.G) + (size_t)cam * Lu.camStride +
                                 (size_t)fRow[r] * Lu.pitch + fCol[c];
            S.fpw[q][r * kFpW + c + 3] = inside(gp, Lu.G, gBytes(R, Lu)) ? ldLevel<kFresh>(gp) : 0u;
        }
        if (last)
            for (int k = threadIdx.x; k < elems; k += kConsumers) {
                const int r = rb + k / kFW, c = k % kFW;
                const uint2* cp = reinterpret_cast<const uint2*>(Lu.C + (size_t)fRow[r] * Lu.pitch + fCol[c]);
                S.cf[r][c + 1] = inside(cp, Lu.C, cBytes(Lu)) ? ldLevel<kFresh>(cp) : make_uint2(0, 0);
            }
    }
}

// The same staging for the tail kernel and k_blend_small, where one unit's
// staging is most of a small level's critical path, so it is kept short in
// instructions and round trips:
//   - every load of the unit is issued into registers before any is stored,
//     so the loads are in flight together;
//   - the footprint rows (G_{j+1} of each camera, then C_{j+1}) are spread
//     over the warps row by row: a row's index mapping is worked out once per
//     row, a lane's two columns once per unit (columns fx0 + lane and, for
//     lanes 0 and 1, fx0 + 32 + lane).
// Threads 0..kConsumers-1; the caller synchronises before the stage is read.
// doG: the cameras' G_j rows, weights and G_{j+1} footprints; doC: the
// C_{j+1} footprint (the only part the previous blend launch writes, so the
// rest may be staged before the wait for it).
template <bool kFresh, class Stage>
__device__ __forceinline__ void stageUnitRows(Stage& S, const RigDev& R, const uint4& raw, int chunk, int half,
                                              bool doG = true, bool doC = true)
{
    constexpr int NC = Stage::kCams;
    constexpr int kWarps = kConsumers / 32;
    constexpr int kGRows = (NC * kFH + kWarps - 1) / kWarps;  // footprint rows of G_{j+1} per warp
    constexpr int kCRows = (kFH + kWarps - 1) / kWarps;       // footprint rows of C_{j+1} per warp
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int lx = lane * 2;
    const int ly = half < 0 ? wp * 2 : 8 * half + wp;
    const int rowsPerThread = half < 0 ? 2 : 1;
    const int j = raw.x & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
    const int tx = raw.y & 0xFFFF, ty = raw.y >> 16;
    const LevelDev& Lj = R.lv[j];
    const bool hasUp = j < R.L;
    const LevelDev& Lu = R.lv[hasUp ? j + 1 : j];
    const int x = tx * kBlendTW + lx, y = ty * kBlendTH + ly;
    const int c0 = chunk * NC;
    const int nc = max(0, min(NC, camCnt - c0));
    const bool last = chunk == unitChunks<NC>(raw) - 1;
    const int fx0 = tx * (kBlendTW / 2) - 1, fy0 = ty * (kBlendTH / 2) - 1;
    const int rb = half < 0 ? 0 : 4 * half, nr = half < 0 ? kFH : 6;
    const int colA = colMap(fx0 + lane, Lu.w);
    const bool hasB = lane < kFW - 32;
    const int colB = hasB ? colMap(fx0 + 32 + lane, Lu.w) : 0;
    uint2 gv[NC][2];
    uint32_t wv[NC][2];
    uint32_t fa[kGRows], fb[kGRows];
    uint2 ca[kCRows], cb[kCRows];
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const int cam = q < nc ? tileCam(raw, R.camLists, c0 + q) : 0;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            gv[q][r] = make_uint2(0, 0);
            wv[q][r] = 0;
            if (doG && q < nc && r < rowsPerThread && y + r < Lj.h) {  // columns up to the pitch are allocated
                const size_t o = (size_t)cam * Lj.camStride + (size_t)(y + r) * Lj.pitch + x;
                const uint2* gp = reinterpret_cast<const uint2*>(Lj.G + o);
                const uint32_t* wp2 = reinterpret_cast<const uint32_t*>(Lj.Wt + o);
                if (inside(gp, Lj.G, gBytes(R, Lj))) gv[q][r] = ldLevel<kFresh>(gp);
                if (inside(wp2, Lj.Wt, wBytes(R, Lj))) wv[q][r] = __ldg(wp2);
            }
        }
    }
    const int gTasks = hasUp && doG ? nc * nr : 0;
#pragma unroll
    for (int i = 0; i < kGRows; i++) {
        const int t = wp + i * kWarps;  // row task: camera t / nr, footprint row rb + t % nr
        fa[i] = fb[i] = 0;
        if (t < gTasks) {
            const int q = t / nr, r = rb + (t - q * nr);
            const uint32_t* row = reinterpret_cast<const uint32_t*>(Lu.G) +
                                  (size_t)tileCam(raw, R.camLists, c0 + q) * Lu.camStride +
                                  (size_t)rowMap(fy0 + r, Lu.h) * Lu.pitch;
            if (inside(row + colA, Lu.G, gBytes(R, Lu))) fa[i] = ldLevel<kFresh>(row + colA);
            if (hasB && inside(row + colB, Lu.G, gBytes(R, Lu))) fb[i] = ldLevel<kFresh>(row + colB);
        }
    }
    const int cTasks = hasUp && last && doC ? nr : 0;
#pragma unroll
    for (int i = 0; i < kCRows; i++) {
        const int t = wp + i * kWarps;
        ca[i] = cb[i] = make_uint2(0, 0);
        if (t < cTasks) {
            const uint2* row = reinterpret_cast<const uint2*>(Lu.C + (size_t)rowMap(fy0 + rb + t, Lu.h) * Lu.pitch);
            if (inside(row + colA, Lu.C, cBytes(Lu))) ca[i] = ldLevel<kFresh>(row + colA);
            if (hasB && inside(row + colB, Lu.C, cBytes(Lu))) cb[i] = ldLevel<kFresh>(row + colB);
        }
    }
#pragma unroll
    for (int q = 0; q < NC; q++)
#pragma unroll
        for (int r = 0; r < 2; r++)
            if (doG && q < nc && r < rowsPerThread) {
                *reinterpret_cast<uint2*>(&S.gj[q][ly + r][lx]) = gv[q][r];
                *reinterpret_cast<uint32_t*>(&S.w[q][ly + r][lx]) = wv[q][r];
            }
#pragma unroll
    for (int i = 0; i < kGRows; i++) {
        const int t = wp + i * kWarps;
        if (t < gTasks) {
            const int q = t / nr, r = rb + (t - q * nr);
            S.fpw[q][r * kFpW + lane + 3] = fa[i];
            if (hasB) S.fpw[q][r * kFpW + 32 + lane + 3] = fb[i];
        }
    }
#pragma unroll
    for (int i = 0; i < kCRows; i++) {
        const int t = wp + i * kWarps;
        if (t < cTasks) {
            S.cf[rb + t][lane + 1] = ca[i];
            if (hasB) S.cf[rb + t][32 + lane + 1] = cb[i];
        }
    }
}

// Accumulate one unit from its stage; at a tile's last unit normalise,
// collapse and store.  Threads 0..kConsumers-1.  staged: the unit came from
// the bulk copies (weights absent for uniform tiles).
//
// Thread (lane, warp) owns rows ly = 2*warp, ly + 1 and columns lx = 2*lane,
// lx + 1 of the tile.  The zero-inserted upsample (weights 1 6 1 for an even
// output row / column, 4 4 for an odd one) reads footprint rows warp ..
// warp+2 (even row: all three; odd row: the last two) and columns lane ..
// lane+2 the same way.
__device__ __forceinline__ void upsample2x2(const uint32_t* g, int pitchW, uint32_t* ulo, uint32_t* uhi)
{
    uint32_t elo[3], ehi[3], olo[3], ohi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint2 a = unpackBytes(g[k]), b = unpackBytes(g[pitchW + k]), c = unpackBytes(g[2 * pitchW + k]);
        elo[k] = a.x + 6 * b.x + c.x;
        ehi[k] = a.y + 6 * b.y + c.y;
        olo[k] = 4 * (b.x + c.x);
        ohi[k] = 4 * (b.y + c.y);
    }
    ulo[0] = elo[0] + 6 * elo[1] + elo[2];
    uhi[0] = ehi[0] + 6 * ehi[1] + ehi[2];
    ulo[1] = 4 * (elo[1] + elo[2]);
    uhi[1] = 4 * (ehi[1] + ehi[2]);
    ulo[2] = olo[0] + 6 * olo[1] + olo[2];
    uhi[2] = ohi[0] + 6 * ohi[1] + ohi[2];
    ulo[3] = 4 * (olo[1] + olo[2]);
    uhi[3] = 4 * (ohi[1] + ohi[2]);
}

// The Laplacian L = G - ((U + 32) >> 6) of one pixel, B and R in the two
// 16-bit lanes of one word, each biased by 256: lanes hold 256 + L in
// 1..511, so neither the lane sums nor the subtraction carry or borrow
// across lanes (U is at most 64 * 255).  G is returned unbiased.
struct Lap {
    uint32_t br;  // (256 + L_B) | (256 + L_R) << 16
    int g;        // L_G
};

__device__ __forceinline__ Lap laplacian(uint32_t gpx, uint32_t ulo, uint32_t uhi)
{
    const uint32_t ubr = ((ulo + 0x00200020u) >> 6) & 0x03FF03FFu;  // round(U) of B and R, per lane
    Lap l;
    l.br = __byte_perm(gpx, 0, 0x4240) + 0x01000100u - ubr;         // G's B and R bytes into the lanes
    l.g = (int)__byte_perm(gpx, 0, 0x4441) - (int)(((uhi & 0xFFFFu) + 32u) >> 6);
    return l;
}

template <class Stage>
__device__ __forceinline__ void computeUnit(const Stage& S, const UnitGeo& G, const uint4& raw, int chunk,
                                            bool staged, BlendAcc& acc)
{
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int lx = 2 * lane, ly = 2 * wp;
    const int j = raw.x & 0xFF, cls = (raw.x >> 8) & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
    const bool uni = ((raw.x >> 24) & kTileUniform) != 0;
    const int tx = raw.y & 0xFFFF, ty = raw.y >> 16;
    const bool hasUp = G.hasUp != 0;
    const int x = tx * kBlendTW + lx, y = ty * kBlendTH + ly;
    const bool active = !(j == 0 && cls == 0);
    constexpr int NC = Stage::kCams;
    const int c0 = chunk * NC;
    const int nc = max(0, min(NC, camCnt - c0));
    const bool first = chunk == 0, last = chunk == unitChunks<NC>(raw) - 1;
    const bool fast = uni && staged;  // weights were not staged
    if (first) {
#pragma unroll
        for (int p = 0; p < 4; p++) {
            acc.r[p][0] = acc.r[p][1] = acc.r[p][2] = 0;
            acc.wsum[p] = 0;
        }
    }
    if (active) {
        for (int q = 0; q < nc; q++) {
            uint32_t ulo[4] = {0, 0, 0, 0}, uhi[4] = {0, 0, 0, 0};
            if (hasUp) upsample2x2(&S.fpw[q][wp * kFpW + 3 + lane], kFpW, ulo, uhi);
            const uint2 gt = *reinterpret_cast<const uint2*>(&S.gj[q][ly][lx]);
            const uint2 gb = *reinterpret_cast<const uint2*>(&S.gj[q][ly + 1][lx]);
            const uint32_t gp[4] = {gt.x, gt.y, gb.x, gb.y};
            uint32_t wq[2] = {0, 0};
            if (!fast) {
                wq[0] = *reinterpret_cast<const uint32_t*>(&S.w[q][ly][lx]);
                wq[1] = *reinterpret_cast<const uint32_t*>(&S.w[q][ly + 1][lx]);
            }
#pragma unroll
            for (int p = 0; p < 4; p++) {
                const Lap l = laplacian(gp[p], ulo[p], uhi[p]);
                if (fast) {
                    acc.r[p][0] = (int)(l.br & 0xFFFFu) - 256;
                    acc.r[p][1] = l.g;
                    acc.r[p][2] = (int)(l.br >> 16) - 256;
                } else {
                    // B and R accumulate w * (256 + L); the 256 * sum(w) comes off at normalisation
                    const int w = (int)((wq[p >> 1] >> (16 * (p & 1))) & 0xFFFFu);
                    acc.r[p][0] += w * (int)(l.br & 0xFFFFu);
                    acc.r[p][1] += w * l.g;
                    acc.r[p][2] += w * (int)(l.br >> 16);
                    acc.wsum[p] += w;
                }
            }
        }
    }
    if (!last) return;
    if (!fast) {
#pragma unroll
        for (int p = 0; p < 4; p++) {
            acc.r[p][0] -= acc.wsum[p] << 8;
            acc.r[p][2] -= acc.wsum[p] << 8;
        }
    }
    int n[4][3];
    if (fast) {
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int c = 0; c < 3; c++) n[p][c] = acc.r[p][c];
    } else if (G.full) {
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int c = 0; c < 3; c++) n[p][c] = (acc.r[p][c] + 128) >> 8;
    } else if (j == 0 && __all_sync(0xffffffffu, ((acc.wsum[0] | acc.wsum[1] | acc.wsum[2] | acc.wsum[3]) & ~256) == 0)) {
        // Level-0 weights are the 0/256 seam masks.  Where each pixel's sum is 0 or 256 (one camera at
        // most: always, unless custom masks overlap), R = 256 L exactly, and R / W truncated is the shift.
#pragma unroll
        for (int p = 0; p < 4; p++)
#pragma unroll
            for (int c = 0; c < 3; c++) n[p][c] = acc.r[p][c] >> 8;
    } else {
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const int d = acc.wsum[p] ? acc.wsum[p] : 1;
            const float inv = __frcp_rn((float)d);
#pragma unroll
            for (int c = 0; c < 3; c++) n[p][c] = divTrunc(acc.r[p][c], d, inv);
        }
    }
    // collapse: + pyrUp32(C_{j+1})
    if (hasUp && active) {
        const uint2* cf = &S.cf[wp][1 + lane];
        int e[3][3], o[3][3];  // vertical sums per footprint column, even / odd row
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint2 a = cf[k], b = cf[kCfW + k], c = cf[2 * kCfW + k];
            const int av[3] = {(short)(a.x & 0xFFFF), (short)(a.x >> 16), (short)(a.y & 0xFFFF)};
            const int bv[3] = {(short)(b.x & 0xFFFF), (short)(b.x >> 16), (short)(b.y & 0xFFFF)};
            const int cv[3] = {(short)(c.x & 0xFFFF), (short)(c.x >> 16), (short)(c.y & 0xFFFF)};
#pragma unroll
            for (int ch = 0; ch < 3; ch++) {
                e[k][ch] = av[ch] + 6 * bv[ch] + cv[ch];
                o[k][ch] = 4 * (bv[ch] + cv[ch]);
            }
        }
#pragma unroll
        for (int ch = 0; ch < 3; ch++) {
            n[0][ch] += (e[0][ch] + 6 * e[1][ch] + e[2][ch] + 32) >> 6;
            n[1][ch] += (4 * (e[1][ch] + e[2][ch]) + 32) >> 6;
            n[2][ch] += (o[0][ch] + 6 * o[1][ch] + o[2][ch] + 32) >> 6;
            n[3][ch] += (4 * (o[1][ch] + o[2][ch]) + 32) >> 6;
        }
    }
    if (j > 0) {
        const long long cext = (long long)G.pitch * G.h * 8;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            if (y + r >= G.h) break;
            short4* Cj = G.C + (size_t)(y + r) * G.pitch + x;
            const int* a = n[2 * r];
            const int* b = n[2 * r + 1];
            if (x + 1 < G.w) {
                if (inside(reinterpret_cast<int4*>(Cj), G.C, cext))
                    *reinterpret_cast<int4*>(Cj) =
                        make_int4((int)((uint32_t)(uint16_t)a[0] | ((uint32_t)(uint16_t)a[1] << 16)),
                                  (int)(uint32_t)(uint16_t)a[2],
                                  (int)((uint32_t)(uint16_t)b[0] | ((uint32_t)(uint16_t)b[1] << 16)),
                                  (int)(uint32_t)(uint16_t)b[2]);
            } else if (x < G.w && inside(Cj, G.C, cext)) {
                Cj[0] = make_short4((short)a[0], (short)a[1], (short)a[2], 0);
            }
        }
        return;
    }
    // level 0 (the render's canvas is even in both directions, the blender's need not be)
    if (y >= G.h || x >= G.w) return;
    const int rows = y + 1 < G.h ? 2 : 1, cols = x + 1 < G.w ? 2 : 1;
    uint32_t o[4] = {0, 0, 0, 0};
    if (cls != 0) {
#pragma unroll
        for (int p = 0; p < 4; p++)
            o[p] = packSatBgr(n[p][0], n[p][1], n[p][2]);
        if (cls == 2) {
            const long long uext = (long long)G.pitch * G.h;
            for (int r = 0; r < rows; r++) {
                const uint8_t* um = G.um + (size_t)(y + r) * G.pitch + x;
                if (!(inside(um, G.um, uext) ? um[0] : 0)) o[2 * r] = 0;
                if (cols == 2 && !(inside(um + 1, G.um, uext) ? um[1] : 0)) o[2 * r + 1] = 0;
            }
        }
    }
    if (G.outFmt == PS_FMT_YUV420P || G.outFmt == PS_FMT_NV12) {  // even sizes only (checked at the API)
        storeYuv(G, x, y, o);
        return;
    }
    const long long oext = G.outPitch * G.h;
    for (int r = 0; r < rows; r++) {
        uint8_t* orow = G.out + (size_t)(y + r) * G.outPitch;
        if (G.outFmt == PS_FMT_BGR32) {
            if (cols == 2 && (reinterpret_cast<uintptr_t>(orow) & 7) == 0) {
                if (inside(reinterpret_cast<uint2*>(orow) + x / 2, G.out, oext))
                    reinterpret_cast<uint2*>(orow)[x / 2] = make_uint2(o[2 * r], o[2 * r + 1]);
            } else {
                if (inside(reinterpret_cast<uint32_t*>(orow) + x, G.out, oext))
                    reinterpret_cast<uint32_t*>(orow)[x] = o[2 * r];
                if (cols == 2 && inside(reinterpret_cast<uint32_t*>(orow) + x + 1, G.out, oext))
                    reinterpret_cast<uint32_t*>(orow)[x + 1] = o[2 * r + 1];
            }
        } else {
            for (int i = 0; i < cols; i++) {
                const uint32_t v = o[2 * r + i];
                if (!insideRange(orow + 3 * (x + i), 3, G.out, oext)) continue;
                orow[3 * (x + i)] = v & 0xFF;
                orow[3 * (x + i) + 1] = (v >> 8) & 0xFF;
                orow[3 * (x + i) + 2] = (v >> 16) & 0xFF;
            }
        }
    }
}

// The tail kernel's variant for levels above 0: one 64x8 half of a tile
// (rows 8*half ..), consumer thread t owning pixels (2*(t%32), t/32) and the
// one to its right, so all eight warps share the few tiles of these levels.
// Same arithmetic as computeUnit; output is the collapsed level C_j.
struct PairAcc {
    int r0[3], r1[3];
    int wsum0, wsum1;
};

template <class Stage>
__device__ __forceinline__ void computeUnitRows(const Stage& S, const UnitGeo& G, const uint4& raw, int chunk,
                                                PairAcc& acc, int half)
{
    const int lx = (threadIdx.x & 31) * 2, lr = threadIdx.x >> 5;  // row in the half tile
    const int ly = 8 * half + lr;                                    // row in the tile
    // vertical taps: even rows footprint rows ly/2 .. ly/2+2 (1 6 1), odd rows
    // (ly+1)/2 .. (ly+1)/2+1 (4 4); footprint columns lx/2 .. lx/2+2 as in computeUnit
    const bool evenRow = (ly & 1) == 0;
    const int vr0 = evenRow ? ly / 2 : (ly + 1) / 2;
    const int fc = lx / 2;
    const int j = raw.x & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
    const int tx = raw.y & 0xFFFF, ty = raw.y >> 16;
    const bool hasUp = G.hasUp != 0;
    const int x = tx * kBlendTW + lx, y = ty * kBlendTH + ly;
    constexpr int NC = Stage::kCams;
    const int c0 = chunk * NC;
    const int nc = max(0, min(NC, camCnt - c0));
    const bool first = chunk == 0, last = chunk == unitChunks<NC>(raw) - 1;
    if (first) {
        acc.r0[0] = acc.r0[1] = acc.r0[2] = acc.r1[0] = acc.r1[1] = acc.r1[2] = 0;
        acc.wsum0 = acc.wsum1 = 0;
    }
    for (int q = 0; q < nc; q++) {
        uint32_t u0lo = 0, u0hi = 0, u1lo = 0, u1hi = 0;
        if (hasUp) {
            const uint32_t* g = &S.fpw[q][0] + 3;
            uint32_t vlo[3], vhi[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const uint2 a = unpackBytes(g[vr0 * kFpW + fc + k]);
                const uint2 b = unpackBytes(g[(vr0 + 1) * kFpW + fc + k]);
                if (evenRow) {
                    const uint2 c = unpackBytes(g[(vr0 + 2) * kFpW + fc + k]);
                    vlo[k] = a.x + 6 * b.x + c.x;
                    vhi[k] = a.y + 6 * b.y + c.y;
                } else {
                    vlo[k] = 4 * (a.x + b.x);
                    vhi[k] = 4 * (a.y + b.y);
                }
            }
            u0lo = vlo[0] + 6 * vlo[1] + vlo[2];
            u0hi = vhi[0] + 6 * vhi[1] + vhi[2];
            u1lo = 4 * (vlo[1] + vlo[2]);
            u1hi = 4 * (vhi[1] + vhi[2]);
        }
        const uint2 gq = *reinterpret_cast<const uint2*>(&S.gj[q][ly][lx]);
        const uint32_t wq = *reinterpret_cast<const uint32_t*>(&S.w[q][ly][lx]);
        const int w0 = (int)(wq & 0xFFFFu), w1 = (int)(wq >> 16);
        // B and R accumulate w * (256 + L); the 256 * sum(w) comes off below
        const Lap l0 = laplacian(gq.x, u0lo, u0hi), l1 = laplacian(gq.y, u1lo, u1hi);
        acc.r0[0] += w0 * (int)(l0.br & 0xFFFFu);
        acc.r0[1] += w0 * l0.g;
        acc.r0[2] += w0 * (int)(l0.br >> 16);
        acc.r1[0] += w1 * (int)(l1.br & 0xFFFFu);
        acc.r1[1] += w1 * l1.g;
        acc.r1[2] += w1 * (int)(l1.br >> 16);
        acc.wsum0 += w0;
        acc.wsum1 += w1;
    }
    if (!last) return;
    acc.r0[0] -= acc.wsum0 << 8;
    acc.r0[2] -= acc.wsum0 << 8;
    acc.r1[0] -= acc.wsum1 << 8;
    acc.r1[2] -= acc.wsum1 << 8;
    int n0[3], n1[3];
    if (G.full) {
#pragma unroll
        for (int c = 0; c < 3; c++) { n0[c] = (acc.r0[c] + 128) >> 8; n1[c] = (acc.r1[c] + 128) >> 8; }
    } else {
        const int d0 = acc.wsum0 ? acc.wsum0 : 1, d1 = acc.wsum1 ? acc.wsum1 : 1;
        const float i0 = __frcp_rn((float)d0), i1 = __frcp_rn((float)d1);
#pragma unroll
        for (int c = 0; c < 3; c++) { n0[c] = divTrunc(acc.r0[c], d0, i0); n1[c] = divTrunc(acc.r1[c], d1, i1); }
    }
    if (hasUp) {
        const uint2* cf = &S.cf[0][0] + 1;
        int v[3][3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint2 a = cf[vr0 * kCfW + fc + k], b = cf[(vr0 + 1) * kCfW + fc + k];
            const int ax = (short)(a.x & 0xFFFF), ay = (short)(a.x >> 16), az = (short)(a.y & 0xFFFF);
            const int bx = (short)(b.x & 0xFFFF), by = (short)(b.x >> 16), bz = (short)(b.y & 0xFFFF);
            if (evenRow) {
                const uint2 c = cf[(vr0 + 2) * kCfW + fc + k];
                v[k][0] = ax + 6 * bx + (short)(c.x & 0xFFFF);
                v[k][1] = ay + 6 * by + (short)(c.x >> 16);
                v[k][2] = az + 6 * bz + (short)(c.y & 0xFFFF);
            } else {
                v[k][0] = 4 * (ax + bx);
                v[k][1] = 4 * (ay + by);
                v[k][2] = 4 * (az + bz);
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            n0[c] += (v[0][c] + 6 * v[1][c] + v[2][c] + 32) >> 6;
            n1[c] += (4 * (v[1][c] + v[2][c]) + 32) >> 6;
        }
    }
    if (y >= G.h || j == 0) return;  // level 0 goes through computeUnit
    short4* Cj = G.C + (size_t)y * G.pitch + x;
    const long long cext = (long long)G.pitch * G.h * 8;
    if (x + 1 < G.w) {
        if (inside(reinterpret_cast<int4*>(Cj), G.C, cext))
            *reinterpret_cast<int4*>(Cj) =
                make_int4((int)((uint32_t)(uint16_t)n0[0] | ((uint32_t)(uint16_t)n0[1] << 16)),
                          (int)(uint32_t)(uint16_t)n0[2],
                          (int)((uint32_t)(uint16_t)n1[0] | ((uint32_t)(uint16_t)n1[1] << 16)),
                          (int)(uint32_t)(uint16_t)n1[2]);
    } else if (x < G.w && inside(Cj, G.C, cext)) {
        Cj[0] = make_short4((short)n0[0], (short)n0[1], (short)n0[2], 0);
    }
}

// Tiles are handed out one at a time through `counter` (zero at launch), so
// a CTA that starts late, behind other frames' kernels, simply takes fewer.
//
// probePolls > 0 is the failure-path test of the bounded waits: consumer
// thread 0 first waits that many polls on an mbarrier that nothing arrives
// on, so the wait runs out, and the timeout is reported as any other
// (status bit 4 of every frame in the launch).
__global__ void __launch_bounds__(kBlendThreads, 4) k_blend(const Segment* __restrict__ gsegs, int nsegs, int total,
                                                            int* __restrict__ counter, int probePolls, int early)
{
    __shared__ BlendStage st[kBStages];
    __shared__ UnitInfo info[kBStages];
    __shared__ uint64_t full[kBStages], empty[kBStages], never;
    __shared__ Segment s_segs[kMaxSmemSegs];
    __shared__ int s_timeout;
    __shared__ int fRow[kFH], fCol[kFW];
    const Segment* segs = gsegs;
    if (nsegs <= kMaxSmemSegs) {
        for (int k = threadIdx.x; k < nsegs; k += kBlendThreads) s_segs[k] = gsegs[k];
        segs = s_segs;
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < kBStages; k++) {
            mbarInit(&full[k], 1);
            mbarInit(&empty[k], kConsumers / 32);
        }
        mbarInit(&never, 1);
        s_timeout = 0;
    }
    if (threadIdx.x < kBStages) info[threadIdx.x].valid = 0;  // a stage read after a wait ran out ends the loop
    __syncthreads();
    const int lane = threadIdx.x & 31;

    if (threadIdx.x >= kConsumers) {
        // ---------------- producer warp ----------------
        // The hand-out counter, items and descriptors are written before the
        // launch sequence, not by a kernel: the first unit is worked out
        // while the previous kernel finishes, and the wait comes before its
        // first copy of level data -- or, with early set (every blend step
        // after the first, where the launch before this one wrote only C
        // levels), before its first copy of C_{j+1}: its G_j, weights and
        // G_{j+1} footprint, written by launches that have completed, are
        // copied (through L2, by the tensor copies) while it finishes.
        bool waited = false;
        auto nextItem = [&] {
            int v = 0;
            if (lane == 0) v = atomicAdd(counter, 1);
            return __shfl_sync(0xffffffffu, v, 0);
        };
        int it = nextItem(), chunk = 0, seg = 0;
        uint4 raw = make_uint4(0, 0, 0, 0);
        bool valid = it < total;
        if (valid) {
            seg = findSegment(segs, nsegs, it, 0);
            raw = __ldg(static_cast<const uint4*>(segs[seg].items) + (it - segs[seg].prefix));
        }
        for (int u = 0;; u++) {
            const int stg = u % kBStages;
            if (u >= kBStages && !mbarWait(&empty[stg], ((u / kBStages) - 1) & 1)) s_timeout = 1;
            UnitInfo ui;
            ui.raw = raw;
            ui.seg = seg;
            ui.chunk = chunk;
            ui.valid = valid;
            ui.staged = 0;
            int nc = 0, cb = 8, j = 0, tx = 0, ty = 0, nCopies = 0;
            bool hasUp = false, last = false, uni = false;
            const RigDev* R = nullptr;
            if (valid) {
                R = segs[seg].rig;
                j = raw.x & 0xFF;
                if (lane == 0) fillGeo(ui.geo, *R, *segs[seg].frame, j);
                const int cls = (raw.x >> 8) & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
                uni = ((raw.x >> 24) & kTileUniform) != 0;
                tx = raw.y & 0xFFFF;
                ty = raw.y >> 16;
                hasUp = j < R->L;
                const LevelDev& Lj = R->lv[j];
                const LevelDev& Lu = R->lv[hasUp ? j + 1 : j];
                nc = max(0, min(kCamsPerUnit, camCnt - chunk * kCamsPerUnit));
                last = chunk == unitChunks(raw) - 1;
                const int fx0 = tx * (kBlendTW / 2) - 1, fy0 = ty * (kBlendTH / 2) - 1;
                const bool rowsIn = (ty + 1) * kBlendTH <= Lj.h;
                const bool fpIn = !hasUp || (fx0 - 3 >= 0 && fx0 - 3 + kFpW <= Lu.w && fy0 >= 0 && fy0 + kFH <= Lu.h);
                const bool active = !(j == 0 && cls == 0);
                if (active && rowsIn && fpIn && (nc > 0 || (hasUp && last))) {
                    ui.staged = 1;
                    cb = kBlendTH + (uni ? 0 : kBlendTH) + (hasUp ? kFH : 0);
                    nCopies = nc * cb + (hasUp && last ? kFH : 0);
                }
            }
            fenceProxyAsync();
            if (lane == 0) info[stg] = ui;
            bool tma = false;
#ifndef PS_CHECK_BOUNDS
            tma = ui.staged && R->tmaps;
#endif
            if (!waited && !(early && tma)) {
                waitPrevGrid();
                allowNextGrid();
                waited = true;
            }
            if (ui.staged) {
                const LevelDev& Lj = R->lv[j];
                const LevelDev& Lu = R->lv[hasUp ? j + 1 : j];
                if (lane == 0) {
                    const uint32_t bytes = nc * (kBlendTH * kBlendTW * 4 + (uni ? 0 : kBlendTH * kBlendTW * 2) +
                                                 (hasUp ? kFH * kFpW * 4 : 0)) +
                                           (hasUp && last ? kFH * kCfW * 8 : 0);
                    mbarArriveExpectTx(&full[stg], bytes);
                }
                __syncwarp();
                const int fx0 = tx * (kBlendTW / 2) - 1, fy0 = ty * (kBlendTH / 2) - 1;
#ifndef PS_CHECK_BOUNDS
                if (R->tmaps) {
                    // one bulk tensor copy per camera and array: the G_j tile,
                    // its weights, its G_{j+1} footprint; then the C_{j+1} footprint
                    if (lane == 0) {
                        const uint8_t* tm = static_cast<const uint8_t*>(R->tmaps);
                        const uint8_t* tmJ = tm + (size_t)j * kTmapsPerLevel * 128;
                        const uint8_t* tmU = tm + (size_t)(j + 1) * kTmapsPerLevel * 128;
                        for (int q = 0; q < nc; q++) {
                            const int cam = tileCam(raw, R->camLists, chunk * kCamsPerUnit + q);
                            tmaLoad3d(&st[stg].gj[q][0][0], tmJ + kTmG * 128, tx * kBlendTW, ty * kBlendTH, cam,
                                      &full[stg]);
                            if (!uni)
                                tmaLoad3d(&st[stg].w[q][0][0], tmJ + kTmW * 128, tx * kBlendTW, ty * kBlendTH, cam,
                                          &full[stg]);
                            if (hasUp) tmaLoad3d(&st[stg].fpw[q][0], tmU + kTmGfp * 128, fx0 - 3, fy0, cam, &full[stg]);
                        }
                    }
                    if (!waited) {  // C_{j+1} is the previous launch's output
                        __syncwarp();
                        waitPrevGrid();
                        allowNextGrid();
                        waited = true;
                    }
                    if (lane == 0 && hasUp && last) {
                        const uint8_t* tmU = static_cast<const uint8_t*>(R->tmaps) + (size_t)(j + 1) * kTmapsPerLevel * 128;
                        tmaLoad2d(&st[stg].cf[0][0], tmU + kTmC * 128, fx0 - 1, fy0, &full[stg]);
                    }
                    nCopies = 0;
                }
#endif
                for (int k = lane; k < nCopies; k += 32) {
                    if (k < nc * cb) {
                        const int q = k / cb;
                        int r = k - q * cb;
                        const int cam = tileCam(raw, R->camLists, chunk * kCamsPerUnit + q);
                        if (r < kBlendTH) {
                            bulkCopyChecked(&st[stg].gj[q][r][0],
                                            Lj.G + (size_t)cam * Lj.camStride + (size_t)(ty * kBlendTH + r) * Lj.pitch +
                                                tx * kBlendTW,
                                            kBlendTW * 4, &full[stg], Lj.G, gBytes(*R, Lj));
                            continue;
                        }
                        r -= kBlendTH;
                        if (!uni) {
                            if (r < kBlendTH) {
                                bulkCopyChecked(&st[stg].w[q][r][0],
                                                Lj.Wt + (size_t)cam * Lj.camStride +
                                                    (size_t)(ty * kBlendTH + r) * Lj.pitch + tx * kBlendTW,
                                                kBlendTW * 2, &full[stg], Lj.Wt, wBytes(*R, Lj));
                                continue;
                            }
                            r -= kBlendTH;
                        }
                        bulkCopyChecked(&st[stg].fpw[q][r * kFpW],
                                        Lu.G + (size_t)cam * Lu.camStride + (size_t)(fy0 + r) * Lu.pitch + (fx0 - 3),
                                        kFpW * 4, &full[stg], Lu.G, gBytes(*R, Lu));
                    } else {
                        const int r = k - nc * cb;
                        bulkCopyChecked(&st[stg].cf[r][0], Lu.C + (size_t)(fy0 + r) * Lu.pitch + (fx0 - 1), kCfW * 8,
                                        &full[stg], Lu.C, cBytes(Lu));
                    }
                }
            } else if (lane == 0) {
                mbarArrive(&full[stg]);
            }
            if (!valid) break;  // the terminal unit is out
            if (chunk + 1 < unitChunks(raw)) {
                chunk++;
            } else {
                chunk = 0;
                it = nextItem();
                valid = it < total;
                if (valid) {
                    seg = findSegment(segs, nsegs, it, seg);
                    raw = __ldg(static_cast<const uint4*>(segs[seg].items) + (it - segs[seg].prefix));
                }
            }
        }
        return;
    }

    // ---------------- consumer warps ----------------
    waitPrevGrid();
    allowNextGrid();
    if (probePolls > 0 && threadIdx.x == 0 && !mbarWait(&never, 0, probePolls)) s_timeout = 1;
    BlendAcc acc;
    for (int u = 0;; u++) {
        const int stg = u % kBStages;
        if (!mbarWait(&full[stg], (u / kBStages) & 1)) s_timeout = 1;
        const UnitInfo& ui = info[stg];  // rewritten only after this warp releases the stage
        const uint4 raw = ui.raw;
        if (!ui.valid) break;
        const int chunk = ui.chunk;
        const bool staged = ui.staged != 0;
        const bool active = !((raw.x & 0xFF) == 0 && ((raw.x >> 8) & 0xFF) == 0);
        if (active && !staged) {
            stageUnitDirect<false>(st[stg], *segs[ui.seg].rig, raw, chunk, fRow, fCol,
                                   [] { namedBarrier(1, kConsumers); });
            namedBarrier(1, kConsumers);
        }
        computeUnit(st[stg], ui.geo, raw, chunk, staged, acc);
        if (active && !staged) fenceProxyAsync();  // our stage writes precede later bulk copies into it
        __syncwarp();
        if (lane == 0) mbarArrive(&empty[stg]);  // this warp is done with the stage
    }
    // The producer's timeouts precede its terminal arrive, which every
    // consumer has waited on; the consumers' own meet here.  A desynchronised
    // ring can have corrupted any unit, so every frame of the launch is flagged.
    namedBarrier(1, kConsumers);
    if (s_timeout && threadIdx.x == 0)
        for (int k = 0; k < nsegs; k++)
            if (segs[k].frame->status) atomicOr(segs[k].frame->status, 4);
}

// ============================================================================
// k_tail: the small top of the pyramid of each rig in one launch.  A cluster
// of 16 CTAs (8 where 16 cannot be co-scheduled) owns one rig: it runs pyrDown levels tailDown..L and
// then blend levels L..tailBlend, spreading each level's tiles over its
// CTAs, with a cluster barrier (release / acquire, so the level's global
// writes are visible to the whole cluster) between levels.  These levels
// hold few tiles, so separate launches would cost mostly launch latency.
// ============================================================================
constexpr int kTailCluster = 8;       // portable cluster size
constexpr int kTailClusterWide = 16;  // used when the GPU can co-schedule it

__device__ __forceinline__ void clusterSync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

union TailSmem {
    DownSmem down;
    BlendStageT<kTailCamsPerUnit> blend;
};

__global__ void __launch_bounds__(kThreads) k_tail(const Segment* __restrict__ segs, int nsegs, int cluster)
{
    extern __shared__ __align__(128) uint8_t tailSmem[];  // a TailSmem (dynamic: above the 48 KB static limit)
    TailSmem& sm = *reinterpret_cast<TailSmem*>(tailSmem);
    
    const int rig = blockIdx.x / cluster, rank = blockIdx.x % cluster;
    initMagic(sm.down.magic);
    waitPrevGrid();
    allowNextGrid();
    if (rig >= nsegs) return;  // never: the grid is nsegs clusters
    __syncthreads();  // the magic table
    const Segment& sg = segs[rig];
    const RigDev& R = *sg.rig;
    for (int J = R.tailDown; J <= R.L; J++) {
        const DownItem* items = R.downItems + R.downOff[J];
        for (int k = rank; k < R.downCnt[J]; k += cluster) pyrDownTile<true>(R, items[k], sm.down);
        clusterSync();
    }
    BlendAcc acc;
    PairAcc pacc;
    for (int j = R.L; j >= R.tailBlend; j--) {
        const BlendItem* items = R.blendItems + R.blendOff[j];
        UnitGeo geo;
        fillGeo(geo, R, *sg.frame, j);
        // levels above 0 (with tailHalf): half tiles with two pixels per
        // thread, so the few tiles of these levels keep twice the CTAs and
        // all warps busy; otherwise whole tiles, 2x2 blocks
        const int parts = j > 0 && R.tailHalf ? 2 : 1;
        for (int k = rank; k < parts * R.blendCnt[j]; k += cluster) {
            const uint4 raw = *reinterpret_cast<const uint4*>(items + k / parts);
            const bool active = !((raw.x & 0xFF) == 0 && ((raw.x >> 8) & 0xFF) == 0);
            for (int chunk = 0; chunk < unitChunks<kTailCamsPerUnit>(raw); chunk++) {
                __syncthreads();  // readers of the previous unit are done
                if (active) stageUnitRows<true>(sm.blend, R, raw, chunk, parts == 2 ? (k & 1) : -1);
                __syncthreads();
                if (parts == 2) computeUnitRows(sm.blend, geo, raw, chunk, pacc, k & 1);
                else computeUnit(sm.blend, geo, raw, chunk, false, acc);
            }
        }
        clusterSync();
    }
}

// ============================================================================
// k_blend_small: blend levels above 0 with few tiles, below the tail.  The
// tail kernel's per-unit code on a plain grid: one 64x8 half tile per work
// item (items 2t and 2t + 1 are the halves of tile t), up to eight cameras
// staged per unit.  In k_blend a CTA walks a tile's cameras two at a time,
// a chain of load-and-compute rounds that these levels cannot hide behind
// other tiles; here each CTA has one short chain and all its warps busy.
// ============================================================================
using SmallStage = BlendStageT<kTailCamsPerUnit>;

__global__ void __launch_bounds__(kThreads) k_blend_small(const Segment* __restrict__ segs, int nsegs, int total,
                                                          int early)
{
    extern __shared__ __align__(128) uint8_t smallSmem[];  // a SmallStage (dynamic: above the 48 KB static limit)
    SmallStage& st = *reinterpret_cast<SmallStage*>(smallSmem);

    // Items and descriptors are written before the launch sequence, not by
    // a kernel: the first item's are read while the previous kernel finishes.
    // With early set (every blend step after the first: the launch before
    // this one wrote only C levels), the first unit's G_j, weights and G_{j+1}
    // footprints, written by launches that have completed, are staged then
    // too, through L2; only its C_{j+1} footprint waits.
    int s = 0;
    uint4 raw = make_uint4(0, 0, 0, 0);
    UnitGeo geo;
    const int first = blockIdx.x;
    const bool pre = early && first < total;
    if (first < total) {
        s = findSegment(segs, nsegs, first, s);
        raw = __ldg(static_cast<const uint4*>(segs[s].items) + ((first - segs[s].prefix) >> 1));
        fillGeo(geo, *segs[s].rig, *segs[s].frame, raw.x & 0xFF);
        if (pre) stageUnitRows<true>(st, *segs[s].rig, raw, 0, (first - segs[s].prefix) & 1, true, false);
    }
    waitPrevGrid();
    allowNextGrid();
    PairAcc acc;
    for (int it = first; it < total; it += gridDim.x) {
        if (it != first) {
            s = findSegment(segs, nsegs, it, s);
            raw = __ldg(static_cast<const uint4*>(segs[s].items) + ((it - segs[s].prefix) >> 1));
            fillGeo(geo, *segs[s].rig, *segs[s].frame, raw.x & 0xFF);
        }
        const Segment& sg = segs[s];
        const RigDev& R = *sg.rig;
        const int half = (it - sg.prefix) & 1;
        for (int chunk = 0; chunk < unitChunks<kTailCamsPerUnit>(raw); chunk++) {
            __syncthreads();  // readers of the previous unit are done
            const bool staged = pre && it == first && chunk == 0;  // G part staged before the wait
            stageUnitRows<false>(st, R, raw, chunk, half, !staged, true);
            __syncthreads();
            computeUnitRows(st, geo, raw, chunk, acc, half);
        }
    }
}

// ============================================================================
// k_cvt_yuv: standalone BGR32 -> YUV420P / NV12 of a device image
// (cvtBGR32ToYUV420P / cvtBGR32ToNV12, ImageProc.cu:97-160).  One thread per
// 2x2 block, consecutive threads on consecutive blocks of a block row.
// ============================================================================
__global__ void __launch_bounds__(kThreads) k_cvt_yuv(const uint8_t* __restrict__ src, long long srcPitch, int w,
                                                      int h, int fmt, uint8_t* __restrict__ py, long long yPitch,
                                                      uint8_t* __restrict__ pu, long long uPitch,
                                                      uint8_t* __restrict__ pv, long long vPitch)
{
    const int bw = w >> 1, bh = h >> 1;
    const long long total = (long long)bw * bh;
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < total;
         b += (long long)gridDim.x * blockDim.x) {
        const int by = (int)(b / bw), bx = (int)(b - (long long)by * bw);
        const int x = bx * 2, y = by * 2;
        const uint32_t* r0 = reinterpret_cast<const uint32_t*>(src + (size_t)y * srcPitch) + x;
        const uint32_t* r1 = reinterpret_cast<const uint32_t*>(src + (size_t)(y + 1) * srcPitch) + x;
        const uint32_t p00 = r0[0], p01 = r0[1], p10 = r1[0], p11 = r1[1];
        uint8_t* y0 = py + (size_t)y * yPitch + x;
        uint8_t* y1 = y0 + yPitch;
        y0[0] = (uint8_t)yuvLuma(p00);
        y0[1] = (uint8_t)yuvLuma(p01);
        y1[0] = (uint8_t)yuvLuma(p10);
        y1[1] = (uint8_t)yuvLuma(p11);
        const int2 c0 = yuvChromaSums(p00), c1 = yuvChromaSums(p10);
        const uint8_t u = (uint8_t)clamp255((c0.x + c1.x) >> (kYuvShift + 1));
        const uint8_t v = (uint8_t)clamp255((c0.y + c1.y) >> (kYuvShift + 1));
        if (fmt == PS_FMT_NV12) {
            pu[(size_t)by * uPitch + x] = u;
            pu[(size_t)by * uPitch + x + 1] = v;
        } else {
            pu[(size_t)by * uPitch + bx] = u;
            pv[(size_t)by * vPitch + bx] = v;
        }
    }
}

// ============================================================================
// k_yuv_to_bgr32: decoder frames YUV420P / NV12 -> BGR32 (cvtYUV420PToBGR32
// / cvtNV12ToBGR32, ImageProc.cu:165-259): per 2x2 block, with u = U - 128,
// v = V - 128 and y' = max(Y - 16, 0) * CY,
//   R = clamp((y' + 2^19 + CVR v) >> 20), G = clamp((y' + 2^19 + CVG v + CUG u) >> 20),
//   B = clamp((y' + 2^19 + CUB u) >> 20)
// (the standard BT.601 studio-range coefficients scaled by 2^20; the shift
// of a negative sum rounds toward minus infinity).  The fourth byte is
// written 0.  One thread per 2x2 block; blockIdx.y is the frame.
// ============================================================================
constexpr int kInvCY = 1220542, kInvCUB = 2116026, kInvCUG = -409993, kInvCVG = -852492, kInvCVR = 1673527;

__device__ __forceinline__ uint32_t yuvPixel(int yv, int ruv, int guv, int buv)
{
    const int yy = max(yv - 16, 0) * kInvCY;
    return packSatBgr((yy + buv) >> kYuvShift, (yy + guv) >> kYuvShift, (yy + ruv) >> kYuvShift);
}

// Eight pixels of a row pair (four 2x2 blocks) per thread: 8-byte luma
// loads, the blocks' chroma in one load, 16-byte stores.
constexpr int kYuvChunks = 2;  // chunks a thread has in flight (4 measured slower)

struct YuvChunk {
    uint2 yt, yb;     // luma of the top and bottom rows
    uint32_t us, vs;  // the four blocks' U and V, one byte each
};

__device__ __forceinline__ YuvChunk yuvLoad(const YuvFrame& F, int cx, int by)
{
    const int x = 8 * cx, y = 2 * by;
    YuvChunk c;
    c.yt = *reinterpret_cast<const uint2*>(F.y + (size_t)y * F.yPitch + x);
    c.yb = *reinterpret_cast<const uint2*>(F.y + (size_t)(y + 1) * F.yPitch + x);
    if (F.fmt == PS_FMT_NV12) {
        const uint2 uv = *reinterpret_cast<const uint2*>(F.u + (size_t)by * F.uPitch + x);
        c.us = __byte_perm(uv.x, uv.y, 0x6420);
        c.vs = __byte_perm(uv.x, uv.y, 0x7531);
    } else {
        c.us = *reinterpret_cast<const uint32_t*>(F.u + (size_t)by * F.uPitch + (x >> 1));
        c.vs = *reinterpret_cast<const uint32_t*>(F.v + (size_t)by * F.vPitch + (x >> 1));
    }
    return c;
}

__device__ __forceinline__ void yuvStore(const YuvFrame& F, int cx, int by, const YuvChunk& c)
{
    const int half = 1 << (kYuvShift - 1);
    uint32_t ot[8], ob[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int u = (int)((c.us >> (8 * k)) & 0xFF) - 128, v = (int)((c.vs >> (8 * k)) & 0xFF) - 128;
        const int ruv = half + kInvCVR * v, guv = half + kInvCVG * v + kInvCUG * u, buv = half + kInvCUB * u;
        const uint32_t wt = k < 2 ? c.yt.x : c.yt.y, wb = k < 2 ? c.yb.x : c.yb.y;
        const int s = 16 * (k & 1);
        ot[2 * k] = yuvPixel((wt >> s) & 0xFF, ruv, guv, buv);
        ot[2 * k + 1] = yuvPixel((wt >> (s + 8)) & 0xFF, ruv, guv, buv);
        ob[2 * k] = yuvPixel((wb >> s) & 0xFF, ruv, guv, buv);
        ob[2 * k + 1] = yuvPixel((wb >> (s + 8)) & 0xFF, ruv, guv, buv);
    }
    const int y = 2 * by;
    uint4* t = reinterpret_cast<uint4*>(F.dst + (size_t)y * F.dstPitch) + 2 * cx;
    uint4* b = reinterpret_cast<uint4*>(F.dst + (size_t)(y + 1) * F.dstPitch) + 2 * cx;
    t[0] = make_uint4(ot[0], ot[1], ot[2], ot[3]);
    t[1] = make_uint4(ot[4], ot[5], ot[6], ot[7]);
    b[0] = make_uint4(ob[0], ob[1], ob[2], ob[3]);
    b[1] = make_uint4(ob[4], ob[5], ob[6], ob[7]);
}

__global__ void __launch_bounds__(kThreads) k_yuv_to_bgr32(YuvFrames f)
{
    const int cam = blockIdx.y;
    const int bw = f.w >> 1, bh = f.h >> 1;
    const YuvFrame& F = f.frame[cam];
    // the launcher takes frames below 2^32 pixels, so 32-bit indices cover the work
    if (F.vec) {
        // kYuvChunks chunks per step, all loaded before any is converted
        const unsigned cw = (unsigned)f.w >> 3;
        const unsigned chunks = cw * (unsigned)bh, stride = gridDim.x * blockDim.x;
        for (unsigned c = blockIdx.x * blockDim.x + threadIdx.x; c < chunks; c += kYuvChunks * stride) {
            YuvChunk v[kYuvChunks];
#pragma unroll
            for (int k = 0; k < kYuvChunks; k++) {
                const unsigned ck = c + k * stride, by = ck / cw;
                if (ck < chunks) v[k] = yuvLoad(F, (int)(ck - by * cw), (int)by);
            }
#pragma unroll
            for (int k = 0; k < kYuvChunks; k++) {
                const unsigned ck = c + k * stride, by = ck / cw;
                if (ck < chunks) yuvStore(F, (int)(ck - by * cw), (int)by, v[k]);
            }
        }
        return;
    }
    const unsigned total = (unsigned)bw * (unsigned)bh;
    for (unsigned b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
        const int by = (int)(b / (unsigned)bw), bx = (int)(b - (unsigned)by * (unsigned)bw);
        const int x = 2 * bx, y = 2 * by;
        const uint8_t* y0 = F.y + (size_t)y * F.yPitch + x;
        const uint8_t* y1 = y0 + F.yPitch;
        int u, v;
        if (F.fmt == PS_FMT_NV12) {
            const uint8_t* c = F.u + (size_t)by * F.uPitch + x;
            u = c[0];
            v = c[1];
        } else {
            u = F.u[(size_t)by * F.uPitch + bx];
            v = F.v[(size_t)by * F.vPitch + bx];
        }
        u -= 128;
        v -= 128;
        const int half = 1 << (kYuvShift - 1);
        const int ruv = half + kInvCVR * v, guv = half + kInvCVG * v + kInvCUG * u, buv = half + kInvCUB * u;
        uint32_t* o0 = reinterpret_cast<uint32_t*>(F.dst + (size_t)y * F.dstPitch) + x;
        uint32_t* o1 = reinterpret_cast<uint32_t*>(F.dst + (size_t)(y + 1) * F.dstPitch) + x;
        const uint32_t p00 = yuvPixel(y0[0], ruv, guv, buv), p01 = yuvPixel(y0[1], ruv, guv, buv);
        const uint32_t p10 = yuvPixel(y1[0], ruv, guv, buv), p11 = yuvPixel(y1[1], ruv, guv, buv);
        if ((F.dstPitch & 7) == 0) {  // x is even, so 8-byte aligned
            *reinterpret_cast<uint2*>(o0) = make_uint2(p00, p01);
            *reinterpret_cast<uint2*>(o1) = make_uint2(p10, p11);
        } else {
            o0[0] = p00;
            o0[1] = p01;
            o1[0] = p10;
            o1[1] = p11;
        }
    }
}

// ---- launch helpers ---------------------------------------------------------
// The lazily computed launch facts below are function-local statics, so
// their first computation is thread-safe (renders may launch from several
// threads).
static int smCount()
{
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return sms;
}

// One wave of `perSm` CTAs per SM, capped by `want` (> 0) and by the work.
static int gridFor(int total, int perSm, int want = 0)
{
    if (want > 0 && want < perSm) perSm = want;
    const int cap = smCount() * perSm;
    return total < cap ? total : cap;
}

// CTAs of `kernel` that fit on one SM (registers, shared memory, threads),
// so a grid of residentPerSm * SMs runs in a single wave; cached per kernel.
template <auto Kernel>
static int residentPerSm(int threads, size_t dynSmem = 0)
{
    static const int cached = [threads, dynSmem] {  // one per kernel
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, Kernel, threads, dynSmem) != cudaSuccess || n < 1) {
            cudaGetLastError();
            n = 1;
        }
        return n;
    }();
    return cached;
}

// Every per-frame kernel is launched with programmatic stream serialisation,
// so its prologue overlaps the previous kernel's tail (see waitPrevGrid).
template <class... Args>
static cudaError_t launchPdl(void (*kernel)(Args...), int grid, int block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

int residentCtasPerSm(int kind)
{
    switch (kind) {
    case 0:
        return std::min(std::min(residentPerSm<k_remap<true, 0>>(kThreads), residentPerSm<k_remap<false, 0>>(kThreads)),
                        std::min(residentPerSm<k_remap<true, PS_FMT_BGR32>>(kThreads),
                                 residentPerSm<k_remap<false, PS_FMT_BGR32>>(kThreads)));
    case 1: return residentPerSm<k_pyrdown>(kThreads);
    case 2: return residentPerSm<k_blend>(kBlendThreads);
    default: return 1;
    }
}

// Entries the launch's tie list has room for.
static int tieListCap(int total)
{
#ifdef PS_CHECK_BOUNDS
    // the checked build's tests may lower it (0: k_remap_fix takes its overflow path)
    static const int perTile = [] {
        const char* v = std::getenv("PS_CHECKED_TIE_LIST_PER_TILE");
        return v ? std::max(0, std::min(std::atoi(v), kRemapTiesPerTile)) : kRemapTiesPerTile;
    }();
    return perTile * total;
#else
    return kRemapTiesPerTile * total;
#endif
}

template <bool kDefer, int kFmt>
static cudaError_t launchRemapAs(const Segment* segs, int nsegs, int total, int perSm, int* counter, int* tieCount,
                                 RemapTie* ties, cudaStream_t st)
{
    return launchPdl(k_remap<kDefer, kFmt>, gridFor(total, residentPerSm<k_remap<kDefer, kFmt>>(kThreads), perSm),
                     kThreads, st, segs, nsegs, total, counter, tieCount, ties, kDefer ? tieListCap(total) : 0);
}

cudaError_t launchRemap(const Segment* segs, int nsegs, int total, int perSm, int* counter, int* tieCount,
                        RemapTie* ties, bool defer, int srcFmt, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    const bool bgr32 = srcFmt == PS_FMT_BGR32;
    if (defer)
        return bgr32 ? launchRemapAs<true, PS_FMT_BGR32>(segs, nsegs, total, perSm, counter, tieCount, ties, st)
                     : launchRemapAs<true, 0>(segs, nsegs, total, perSm, counter, tieCount, ties, st);
    return bgr32 ? launchRemapAs<false, PS_FMT_BGR32>(segs, nsegs, total, perSm, counter, tieCount, ties, st)
                 : launchRemapAs<false, 0>(segs, nsegs, total, perSm, counter, tieCount, ties, st);
}

cudaError_t launchRemapFix(const Segment* segs, int nsegs, int total, const int* tieCount, const RemapTie* ties,
                           cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_remap_fix, 2 * smCount(), kThreads, st, segs, nsegs, total, tieCount, ties,
                     tieListCap(total));
}

cudaError_t launchPyrDown(const Segment* segs, int nsegs, int total, int perSm, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_pyrdown, gridFor(total, residentPerSm<k_pyrdown>(kThreads), perSm), kThreads, st, segs, nsegs,
                     total);
}

cudaError_t launchLinear(const Segment* segs, int nsegs, int total, int maxCams, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(gridFor(total, residentPerSm<k_linear>(kThreads, (size_t)PS_MAX_CAMS * 768)));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = (size_t)maxCams * 768;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_linear, segs, nsegs, total);
}

cudaError_t launchBlend(const Segment* segs, int nsegs, int total, int perSm, int* counter, int probePolls,
                        bool early, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_blend, gridFor(total, residentPerSm<k_blend>(kBlendThreads), perSm), kBlendThreads, st, segs,
                     nsegs, total, counter, probePolls, (int)early);
}

cudaError_t launchBlendSmall(const Segment* segs, int nsegs, int total, bool early, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    static const int perSm = [] {  // the attribute is set before any launch can see perSm
        cudaFuncSetAttribute(k_blend_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmallStage));
        return residentPerSm<k_blend_small>(kThreads, sizeof(SmallStage));
    }();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(gridFor(total, perSm));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = sizeof(SmallStage);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_blend_small, segs, nsegs, total, (int)early);
}

int tailClusterMax()
{
    static const int widest = [] {  // the attributes are set before any launch can see the width
        int size = kTailCluster;
        cudaFuncSetAttribute(k_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TailSmem));
        if (cudaFuncSetAttribute(k_tail, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(kTailClusterWide);
            cfg.blockDim = dim3(kThreads);
            cfg.dynamicSmemBytes = sizeof(TailSmem);
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = kTailClusterWide;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, k_tail, &cfg) == cudaSuccess && clusters >= 1)
                size = kTailClusterWide;
        }
        cudaGetLastError();
        return size;
    }();
    return widest;
}

cudaError_t launchTail(const Segment* segs, int nsegs, int cluster, cudaStream_t st)
{
    if (nsegs <= 0) return cudaSuccess;
    const int widest = tailClusterMax();
    if (cluster <= 0 || cluster > widest) cluster = widest;
    else cluster = cluster >= kTailClusterWide ? kTailClusterWide : kTailCluster;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nsegs * cluster);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = sizeof(TailSmem);
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cudaLaunchKernelEx(&cfg, k_tail, segs, nsegs, cluster);
}

cudaError_t launchCvtYuv(const uint8_t* src, long long srcPitch, int w, int h, int fmt, uint8_t* y, long long yPitch,
                         uint8_t* u, long long uPitch, uint8_t* v, long long vPitch, cudaStream_t st)
{
    const long long blocks = (long long)(w / 2) * (h / 2);
    if (blocks <= 0) return cudaSuccess;
    const int grid = (int)std::min<long long>((blocks + kThreads - 1) / kThreads, (long long)smCount() * 8);
    k_cvt_yuv<<<grid, kThreads, 0, st>>>(src, srcPitch, w, h, fmt, y, yPitch, u, uPitch, v, vPitch);
    return cudaGetLastError();
}

// Frames whose width and planes allow the 8-pixel path.
static bool yuvVector(const YuvFrame& F, int w)
{
    auto al = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; };
    if (w % 8 || !al(F.y, 8) || F.yPitch % 8) return false;
    if (F.fmt == PS_FMT_NV12) {
        if (!al(F.u, 8) || F.uPitch % 8) return false;
    } else if (!al(F.u, 4) || F.uPitch % 4 || !al(F.v, 4) || F.vPitch % 4) {
        return false;
    }
    return al(F.dst, 16) && F.dstPitch % 16 == 0;
}

cudaError_t launchYuvToBgr32(const YuvFrames& frames, cudaStream_t st)
{
    if (frames.n <= 0 || frames.w <= 0 || frames.h <= 0) return cudaSuccess;
    if ((long long)frames.w * frames.h >= (1LL << 32)) return cudaErrorInvalidValue;
    YuvFrames f = frames;
    for (int i = 0; i < f.n; i++) f.frame[i].vec = yuvVector(f.frame[i], f.w) ? 1 : 0;
    // work items per frame: 2x2 blocks, or 8x2 chunks (kYuvChunks per thread) on the vector path
    bool vec = true;
    for (int i = 0; i < f.n; i++) vec = vec && f.frame[i].vec;
    const long long items = vec ? ((long long)(f.w / 8) * (f.h / 2) + kYuvChunks - 1) / kYuvChunks
                                : (long long)(f.w / 2) * (f.h / 2);
    // one wave of 8 CTAs per SM across all frames, or fewer CTAs if the work is smaller
    const long long want = std::max<long long>(1, (long long)smCount() * 8 / f.n);
    const int gx = (int)std::min<long long>((items + kThreads - 1) / kThreads, want);
    k_yuv_to_bgr32<<<dim3(gx, f.n), kThreads, 0, st>>>(f);
    return cudaGetLastError();
}

cudaError_t launchReprojectTo16S(const uint8_t* src, long long srcPitch, int srcW, int srcH, int srcFmt,
                                 const float* xmap, const float* ymap, long long mapPitch, int dstW, int dstH,
                                 const uint8_t* lut, int16_t* dst, long long dstPitch, cudaStream_t st)
{
    dim3 grid((dstW + 31) / 32, (dstH + 7) / 8);
    k_reproject16s<<<grid, kThreads, 0, st>>>(src, srcPitch, srcW, srcH, srcFmt, xmap, ymap, mapPitch, dstW, dstH,
                                              lut, reinterpret_cast<short4*>(dst), dstPitch);
    return cudaGetLastError();
}

}  // namespace ps

// ---- the checked build's counter ------------------------------------------------
namespace ps {
long long boundsViolations(bool reset)
{
#ifdef PS_CHECK_BOUNDS
    unsigned long long v = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return -2;  // the renders run on their own streams
    if (cudaMemcpyFromSymbol(&v, g_boundsViolations, sizeof v) != cudaSuccess) return -2;
    if (reset) {
        const unsigned long long z = 0;
        if (cudaMemcpyToSymbol(g_boundsViolations, &z, sizeof z) != cudaSuccess) return -2;
    }
    return (long long)v;
#else
    (void)reset;
    return -1;
#endif
}
}  // namespace ps
