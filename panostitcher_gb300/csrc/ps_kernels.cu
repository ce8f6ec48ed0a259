// ps_kernels.cu -- the per-frame stitch kernels (sm_103a).
//
// One frame of one or more rigs runs as 2L+2 launches over prepared work
// lists:
//   k_remap        level 0: LUT gain + bilinear remap of every covered tile,
//                  written as uchar4 G0 (cudaTransform + cudaReprojectTo16S);
//   k_pyrdown      levels 1..L: masked 5x5 decimation G_j -> G_{j+1}
//                  (pyrDown16SC4To16SC4 with alpha scale);
//   k_blend        levels L..0: for every canvas tile, the Laplacian of each
//                  camera whose seam weight touches the tile
//                  (G_j - pyrUp(G_{j+1})), its weighted accumulation, the
//                  normalisation, and the collapse step pyrUp(C_{j+1}) + N_j,
//                  all in registers; level 0 writes the 8-bit output with
//                  the uncovered pixels zeroed.
// The reference runs the same arithmetic as ~35 launches per camera plus
// ~36 per frame over full-canvas int16/int32 images
// (source/CudaAccel/CudaMultibandBlend.cpp:785-823).
#include "ps_device.cuh"
#include "ps_internal.h"

namespace ps {

__constant__ int c_k5[5] = {1, 4, 6, 4, 1};

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
__device__ __forceinline__ uint32_t loadTexel(const uint8_t* row, int x, int fmt)
{
    if (fmt == PS_FMT_BGR32) return __ldg(reinterpret_cast<const uint32_t*>(row) + x);
    const uint8_t* p = row + 3 * x;
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

// Returns B | G << 8 | R << 16 (0 where the map is invalid).
__device__ __forceinline__ uint32_t remapPixel(float2 m, const uint8_t* base, long long pitch, int fmt, int sw,
                                               int sh, const uint8_t* lut)
{
    if (!(m.x >= 0.f && m.y >= 0.f && m.x < (float)sw && m.y < (float)sh)) return 0;
    const int x0 = (int)m.x, y0 = (int)m.y;
    const int x1 = min(x0 + 1, sw - 1), y1 = min(y0 + 1, sh - 1);
    const uint8_t* r0 = base + (size_t)y0 * pitch;
    const uint8_t* r1 = base + (size_t)y1 * pitch;
    const uint32_t t00 = loadTexel(r0, x0, fmt), t01 = loadTexel(r0, x1, fmt);
    const uint32_t t10 = loadTexel(r1, x0, fmt), t11 = loadTexel(r1, x1, fmt);
    const float fx = m.x - (float)x0, fy = m.y - (float)y0;
    const float gx = 1.f - fx, gy = 1.f - fy;
    const float w00 = gx * gy, w01 = fx * gy, w10 = gx * fy, w11 = fx * fy;
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int s = 8 * c;
        const int p00 = lut[c * 256 + ((t00 >> s) & 0xFF)];
        const int p01 = lut[c * 256 + ((t01 >> s) & 0xFF)];
        const int p10 = lut[c * 256 + ((t10 >> s) & 0xFF)];
        const int p11 = lut[c * 256 + ((t11 >> s) & 0xFF)];
        const float r = fmaf((float)p11, w11, fmaf((float)p10, w10, fmaf((float)p01, w01, (float)p00 * w00)));
        int v;
        if (fabsf(r - floorf(r) - 0.5f) < 2e-4f)
            v = bilinearExact((double)m.x, (double)m.y, x0, y0, p00, p01, p10, p11);
        else
            v = min(max(__float2int_rn(r), 0), 255);
        out |= (uint32_t)v << s;
    }
    return out;
}

// Level-0 remap over the covered 32x16 tiles of every camera; each thread
// remaps two pixels (rows ly and ly + 8) so two independent gathers are in
// flight; the tile's map is 512 consecutive float2.
__global__ void __launch_bounds__(kThreads) k_remap(const Segment* __restrict__ segs, int nsegs, int total)
{
    __shared__ uint8_t lut[3 * 256];
    long long loaded = -1;
    int s = 0, begin, end;
    itemRange(total, begin, end);
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    waitPrevGrid();
    allowNextGrid();
    for (int it = begin; it < end; it++) {
        s = findSegment(segs, nsegs, it, s);
        const Segment sg = segs[s];
        const RemapItem item = static_cast<const RemapItem*>(sg.items)[it - sg.prefix];
        const FrameDev& F = *sg.frame;
        const RigDev& R = *sg.rig;
        const float2* mt = R.maps + (size_t)item.mapTile * (kRemapTW * kRemapTH);
        const float2 m0 = __ldg(mt + threadIdx.x), m1 = __ldg(mt + threadIdx.x + kThreads);
        const long long key = ((long long)s << 16) | item.cam;
        if (key != loaded) {  // uniform across the block
            __syncthreads();
            const uint8_t* src = F.luts + item.cam * 768;
            for (int k = threadIdx.x; k < 768; k += kThreads) lut[k] = __ldg(src + k);
            __syncthreads();
            loaded = key;
        }
        const int x = item.tx * kRemapTW + lx, y0 = item.ty * kRemapTH + ly, y1 = y0 + 8;
        const uint8_t* base = F.src[item.cam];
        const long long pitch = F.srcPitch[item.cam];
        const uint32_t v0 = remapPixel(m0, base, pitch, F.srcFmt, R.srcW, R.srcH, lut);
        const uint32_t v1 = remapPixel(m1, base, pitch, F.srcFmt, R.srcW, R.srcH, lut);
        const LevelDev& L0 = R.lv[0];
        uint32_t* G = reinterpret_cast<uint32_t*>(L0.G) + (size_t)item.cam * L0.camStride + x;
        if (x < R.W) {
            if (y0 < R.H) G[(size_t)y0 * L0.pitch] = v0;
            if (y1 < R.H) G[(size_t)y1 * L0.pitch] = v1;
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
// One CTA produces a 32x16 output tile from a 67x35 input tile staged in
// shared memory; the separable passes add two channels per 32-bit word.
// ============================================================================
constexpr int kDInW = 2 * kDownTW + 3;   // 67
constexpr int kDInH = 2 * kDownTH + 3;   // 35

constexpr int kDLoads = (kDInH * kDInW + kThreads - 1) / kThreads;   // 10 tile elements per thread

__global__ void __launch_bounds__(kThreads) k_pyrdown(const Segment* __restrict__ segs, int nsegs, int total)
{
    __shared__ uint32_t s_in[kDInH][kDInW];
    __shared__ uint2 s_v[kDownTH][kDInW];
    __shared__ uint32_t s_magic[257];
    for (int m = threadIdx.x; m < 257; m += kThreads) s_magic[m] = m ? (uint32_t)((16777216u + m - 1) / m) : 0u;
    int s = 0, begin, end;
    itemRange(total, begin, end);
    const int ox = threadIdx.x & 31, oy = threadIdx.x >> 5;
    waitPrevGrid();
    allowNextGrid();
    for (int it = begin; it < end; it++) {
        s = findSegment(segs, nsegs, it, s);
        const Segment sg = segs[s];
        const DownItem item = static_cast<const DownItem*>(sg.items)[it - sg.prefix];
        const RigDev& R = *sg.rig;
        const LevelDev& Ls = R.lv[item.level - 1];
        const LevelDev& Ld = R.lv[item.level];
        const int sw = Ls.w, sh = Ls.h;
        const int ox0 = item.tx * kDownTW, oy0 = item.ty * kDownTH;
        const int ix0 = 2 * ox0 - 2, iy0 = 2 * oy0 - 2;
        const uint32_t* G = reinterpret_cast<const uint32_t*>(Ls.G) + (size_t)item.cam * Ls.camStride;
        // issue every load of the item before the first barrier: the tile and the two divisors
        const int X = ox0 + ox, Y0 = oy0 + oy, Y1 = Y0 + 8;
        const size_t o0 = (size_t)item.cam * Ld.camStride + (size_t)Y0 * Ld.pitch + X;
        const size_t o1 = o0 + (size_t)8 * Ld.pitch;
        const bool ok0 = X < Ld.w && Y0 < Ld.h, ok1 = X < Ld.w && Y1 < Ld.h;
        const int m0 = ok0 ? __ldg(Ld.Am + o0) : 0, m1 = ok1 ? __ldg(Ld.Am + o1) : 0;
        uint32_t v[kDLoads];
        const bool interior = ix0 >= 0 && iy0 >= 0 && ix0 + kDInW <= sw && iy0 + kDInH <= sh;
#pragma unroll
        for (int q = 0; q < kDLoads; q++) {
            const int k = threadIdx.x + q * kThreads;
            if (k < kDInH * kDInW) {
                const int r = k / kDInW, c = k - r * kDInW;
                const int gy = interior ? iy0 + r : rowMap(iy0 + r, sh);
                const int gx = interior ? ix0 + c : colMap(ix0 + c, sw);
                v[q] = __ldg(G + (size_t)gy * Ls.pitch + gx);
            }
        }
        __syncthreads();  // the previous item's readers are done with shared memory
#pragma unroll
        for (int q = 0; q < kDLoads; q++) {
            const int k = threadIdx.x + q * kThreads;
            if (k < kDInH * kDInW) (&s_in[0][0])[k] = v[q];
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kDownTH * kDInW; k += kThreads) {
            const int r = k / kDInW, c = k - r * kDInW;
            uint32_t lo = 0, hi = 0;
#pragma unroll
            for (int t = 0; t < 5; t++) {
                const uint2 p = unpackBytes(s_in[2 * r + t][c]);
                lo += c_k5[t] * p.x;
                hi += c_k5[t] * p.y;
            }
            s_v[r][c] = make_uint2(lo, hi);
        }
        __syncthreads();
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int r = oy + 8 * half;
            uint32_t lo = 0, hi = 0;
#pragma unroll
            for (int t = 0; t < 5; t++) {
                const uint2 q = s_v[r][2 * ox + t];
                lo += c_k5[t] * q.x;
                hi += c_k5[t] * q.y;
            }
            const int m = half ? m1 : m0;
            uint32_t outv = 0;
            if (m) {
                const unsigned long long mg = s_magic[m];
                const uint32_t b = (uint32_t)(((lo & 0xFFFFu) * mg) >> 24);
                const uint32_t rr = (uint32_t)(((lo >> 16) * mg) >> 24);
                const uint32_t g = (uint32_t)(((hi & 0xFFFFu) * mg) >> 24);
                outv = b | (g << 8) | (rr << 16);
            }
            if (half ? ok1 : ok0) reinterpret_cast<uint32_t*>(Ld.G)[half ? o1 : o0] = outv;
        }
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
// A CTA covers a 64x8 tile; thread t owns pixels (2*(t%32), t/32) and the
// one to its right.  Every global load of a tile (the C_{j+1} footprint, the
// G_{j+1} footprints of two cameras at a time, their weights and G_j pixels) is
// issued before one barrier, so a tile costs one memory round trip; the next
// tile's descriptor is prefetched meanwhile.
// ============================================================================
constexpr int kFW = kBlendTW / 2 + 2;  // 34
constexpr int kFH = kBlendTH / 2 + 2;  // 6
constexpr int kFElems = kFW * kFH;     // 204
constexpr int kCamsPerPass = 2;
constexpr int kFLoads = (kCamsPerPass * kFElems + kThreads - 1) / kThreads;  // 4
constexpr int kMaxSmemSegs = 64;

// q-th camera of a blend tile (raw 16-byte descriptor)
__device__ __forceinline__ int tileCam(const uint4& raw, const uint8_t* camLists, int q)
{
    if (((raw.x >> 16) & 0xFF) > kInlineCams) return __ldg(camLists + raw.z + q);
    const uint32_t w = q < 4 ? raw.z : raw.w;
    return (int)((w >> (8 * (q & 3))) & 0xFF);
}

__global__ void __launch_bounds__(kThreads, 4) k_blend(const Segment* __restrict__ gsegs, int nsegs, int total)
{
    __shared__ uint32_t s_g[kCamsPerPass * kFElems];
    __shared__ int4 s_c[kFElems];
    __shared__ Segment s_segs[kMaxSmemSegs];
    const Segment* segs = gsegs;
    if (nsegs <= kMaxSmemSegs) {
        for (int k = threadIdx.x; k < nsegs; k += kThreads) s_segs[k] = gsegs[k];
        __syncthreads();
        segs = s_segs;
    }
    const int lx = (threadIdx.x & 31) * 2, ly = threadIdx.x >> 5;
    // vertical taps of the zero-inserted upsample for this row's parity:
    // even rows take footprint rows ly/2 .. ly/2+2 with weights 1 6 1,
    // odd rows (ly+1)/2 .. (ly+1)/2+1 with weights 4 4
    const bool evenRow = (ly & 1) == 0;
    const int vr0 = evenRow ? ly / 2 : (ly - 1) / 2 + 1;
    // footprint columns: even pixel lx/2 .. lx/2+2 (1 6 1), odd pixel lx/2+1 .. lx/2+2 (4 4)
    const int fc = lx / 2;
    // interleaved tiles balance the load (uncovered bands are cheap, seams are not)
    int s = 0;
    uint4 nextRaw = make_uint4(0, 0, 0, 0);
    if ((int)blockIdx.x < total) {
        s = findSegment(segs, nsegs, blockIdx.x, 0);
        nextRaw = __ldg(static_cast<const uint4*>(segs[s].items) + (blockIdx.x - segs[s].prefix));
    }
    waitPrevGrid();
    allowNextGrid();
    for (int it = blockIdx.x; it < total; it += gridDim.x) {
        const uint4 raw = nextRaw;
        const int cs = s;
        const int nx = it + (int)gridDim.x;
        if (nx < total) {
            s = findSegment(segs, nsegs, nx, s);
            nextRaw = __ldg(static_cast<const uint4*>(segs[s].items) + (nx - segs[s].prefix));
        }
        const Segment& sg = segs[cs];
        const RigDev& R = *sg.rig;
        const int j = raw.x & 0xFF, cls = (raw.x >> 8) & 0xFF, camCnt = (raw.x >> 16) & 0xFF;
        const int tx = raw.y & 0xFFFF, ty = raw.y >> 16;
        const LevelDev& Lj = R.lv[j];
        const int x = tx * kBlendTW + lx, y = ty * kBlendTH + ly;
        const bool rowOk = y < Lj.h;
        const bool active = !(j == 0 && cls == 0);
        const bool hasUp = j < R.L;
        const LevelDev& Lu = R.lv[hasUp ? j + 1 : j];
        const int fx0 = tx * (kBlendTW / 2) - 1, fy0 = ty * (kBlendTH / 2) - 1;
        const bool interiorU = fx0 >= 0 && fy0 >= 0 && fx0 + kFW <= Lu.w && fy0 + kFH <= Lu.h;
        int r0[3] = {0, 0, 0}, r1[3] = {0, 0, 0};
        int wsum0 = 0, wsum1 = 0;

        if (active) {
            // collapse footprint of C_{j+1}: issued first, staged with the first pass
            short4 cv = make_short4(0, 0, 0, 0);
            if (hasUp && threadIdx.x < kFElems) {
                const int r = threadIdx.x / kFW, c = threadIdx.x - r * kFW;
                const int gy = interiorU ? fy0 + r : rowMap(fy0 + r, Lu.h);
                const int gx = interiorU ? fx0 + c : colMap(fx0 + c, Lu.w);
                cv = Lu.C[(size_t)gy * Lu.pitch + gx];
            }
            for (int c0 = 0;; c0 += kCamsPerPass) {
                const int nc = min(kCamsPerPass, camCnt - c0);
                uint32_t fv[kFLoads];
                if (hasUp) {
#pragma unroll
                    for (int q = 0; q < kFLoads; q++) {
                        const int k = threadIdx.x + q * kThreads;
                        if (k < nc * kFElems) {
                            const int cq = k / kFElems, e = k - cq * kFElems;
                            const int r = e / kFW, c = e - r * kFW;
                            const int cam = tileCam(raw, R.camLists, c0 + cq);
                            const int gy = interiorU ? fy0 + r : rowMap(fy0 + r, Lu.h);
                            const int gx = interiorU ? fx0 + c : colMap(fx0 + c, Lu.w);
                            fv[q] = __ldg(reinterpret_cast<const uint32_t*>(Lu.G) + (size_t)cam * Lu.camStride +
                                          (size_t)gy * Lu.pitch + gx);
                        }
                    }
                }
                uint32_t wp[kCamsPerPass];
                uint2 gp[kCamsPerPass];
#pragma unroll
                for (int q = 0; q < kCamsPerPass; q++) {
                    wp[q] = 0;
                    gp[q] = make_uint2(0, 0);
                    if (q < nc && rowOk) {
                        const int cam = tileCam(raw, R.camLists, c0 + q);
                        const size_t o = (size_t)cam * Lj.camStride + (size_t)y * Lj.pitch + x;
                        wp[q] = __ldg(reinterpret_cast<const uint32_t*>(Lj.Wt + o));
                        gp[q] = __ldg(reinterpret_cast<const uint2*>(Lj.G + o));
                    }
                }
                if (hasUp) {
                    __syncthreads();  // readers of the previous pass / tile are done
#pragma unroll
                    for (int q = 0; q < kFLoads; q++) {
                        const int k = threadIdx.x + q * kThreads;
                        if (k < nc * kFElems) s_g[k] = fv[q];
                    }
                    if (c0 == 0 && threadIdx.x < kFElems) s_c[threadIdx.x] = make_int4(cv.x, cv.y, cv.z, 0);
                    __syncthreads();
                }
#pragma unroll
                for (int q = 0; q < kCamsPerPass; q++) {
                    if (q >= nc) break;
                    uint32_t u0lo = 0, u0hi = 0, u1lo = 0, u1hi = 0;
                    if (hasUp) {
                        const uint32_t* g = s_g + q * kFElems;
                        uint32_t vlo[3], vhi[3];
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            const uint2 a = unpackBytes(g[vr0 * kFW + fc + k]);
                            const uint2 b = unpackBytes(g[(vr0 + 1) * kFW + fc + k]);
                            if (evenRow) {
                                const uint2 c = unpackBytes(g[(vr0 + 2) * kFW + fc + k]);
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
                    const int w0 = (int)(wp[q] & 0xFFFFu), w1 = (int)(wp[q] >> 16);
                    const uint2 gq = gp[q];
                    // L = G - ((U + 32) >> 6), per channel
                    r0[0] += w0 * ((int)(gq.x & 0xFF) - (int)(((u0lo & 0xFFFFu) + 32) >> 6));
                    r0[1] += w0 * ((int)((gq.x >> 8) & 0xFF) - (int)(((u0hi & 0xFFFFu) + 32) >> 6));
                    r0[2] += w0 * ((int)((gq.x >> 16) & 0xFF) - (int)(((u0lo >> 16) + 32) >> 6));
                    r1[0] += w1 * ((int)(gq.y & 0xFF) - (int)(((u1lo & 0xFFFFu) + 32) >> 6));
                    r1[1] += w1 * ((int)((gq.y >> 8) & 0xFF) - (int)(((u1hi & 0xFFFFu) + 32) >> 6));
                    r1[2] += w1 * ((int)((gq.y >> 16) & 0xFF) - (int)(((u1lo >> 16) + 32) >> 6));
                    wsum0 += w0;
                    wsum1 += w1;
                }
                if (c0 + kCamsPerPass >= camCnt) break;
            }
        }
        // normalise
        int n0[3], n1[3];
        if (R.full) {
#pragma unroll
            for (int c = 0; c < 3; c++) { n0[c] = (r0[c] + 128) >> 8; n1[c] = (r1[c] + 128) >> 8; }
        } else {
            const int d0 = wsum0 ? wsum0 : 1, d1 = wsum1 ? wsum1 : 1;
            const float i0 = __frcp_rn((float)d0), i1 = __frcp_rn((float)d1);
#pragma unroll
            for (int c = 0; c < 3; c++) { n0[c] = divTrunc(r0[c], d0, i0); n1[c] = divTrunc(r1[c], d1, i1); }
        }
        // collapse: + pyrUp32(C_{j+1}), from the footprint staged above
        if (hasUp && active) {
            int v[3][3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const int4 a = s_c[vr0 * kFW + fc + k];
                const int4 b = s_c[(vr0 + 1) * kFW + fc + k];
                if (evenRow) {
                    const int4 c = s_c[(vr0 + 2) * kFW + fc + k];
                    v[k][0] = a.x + 6 * b.x + c.x;
                    v[k][1] = a.y + 6 * b.y + c.y;
                    v[k][2] = a.z + 6 * b.z + c.z;
                } else {
                    v[k][0] = 4 * (a.x + b.x);
                    v[k][1] = 4 * (a.y + b.y);
                    v[k][2] = 4 * (a.z + b.z);
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                n0[c] += (v[0][c] + 6 * v[1][c] + v[2][c] + 32) >> 6;
                n1[c] += (4 * (v[1][c] + v[2][c]) + 32) >> 6;
            }
        }
        if (!rowOk) continue;
        if (j > 0) {
            short4* Cj = Lj.C + (size_t)y * Lj.pitch + x;
            if (x + 1 < Lj.w) {
                *reinterpret_cast<int4*>(Cj) = make_int4(
                    (int)((uint32_t)(uint16_t)n0[0] | ((uint32_t)(uint16_t)n0[1] << 16)), (int)(uint32_t)(uint16_t)n0[2],
                    (int)((uint32_t)(uint16_t)n1[0] | ((uint32_t)(uint16_t)n1[1] << 16)), (int)(uint32_t)(uint16_t)n1[2]);
            } else if (x < Lj.w) {
                Cj[0] = make_short4((short)n0[0], (short)n0[1], (short)n0[2], 0);
            }
        } else {
            const FrameDev& F = *sg.frame;
            uint32_t o0 = 0, o1 = 0;
            if (cls != 0) {
                o0 = (uint32_t)min(max(n0[0], 0), 255) | ((uint32_t)min(max(n0[1], 0), 255) << 8) |
                     ((uint32_t)min(max(n0[2], 0), 255) << 16);
                o1 = (uint32_t)min(max(n1[0], 0), 255) | ((uint32_t)min(max(n1[1], 0), 255) << 8) |
                     ((uint32_t)min(max(n1[2], 0), 255) << 16);
                if (cls == 2) {
                    const uint8_t* um = R.unionMask + (size_t)y * Lj.pitch + x;
                    if (!um[0]) o0 = 0;
                    if (x + 1 < Lj.w && !um[1]) o1 = 0;
                }
            }
            uint8_t* orow = F.out + (size_t)y * F.outPitch;
            if (F.outFmt == PS_FMT_BGR32) {
                if (x + 1 < Lj.w && ((reinterpret_cast<uintptr_t>(orow) & 7) == 0)) {
                    reinterpret_cast<uint2*>(orow)[x / 2] = make_uint2(o0, o1);
                } else {
                    if (x < Lj.w) reinterpret_cast<uint32_t*>(orow)[x] = o0;
                    if (x + 1 < Lj.w) reinterpret_cast<uint32_t*>(orow)[x + 1] = o1;
                }
            } else {
                if (x < Lj.w) {
                    orow[3 * x] = o0 & 0xFF;
                    orow[3 * x + 1] = (o0 >> 8) & 0xFF;
                    orow[3 * x + 2] = (o0 >> 16) & 0xFF;
                }
                if (x + 1 < Lj.w) {
                    orow[3 * x + 3] = o1 & 0xFF;
                    orow[3 * x + 4] = (o1 >> 8) & 0xFF;
                    orow[3 * x + 5] = (o1 >> 16) & 0xFF;
                }
            }
        }
    }
}

// ---- launch helpers ---------------------------------------------------------
static int smCount()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms = v > 0 ? v : 1;
    }
    return sms;
}

static int gridFor(int total, int perSm)
{
    const int cap = smCount() * perSm;
    return total < cap ? total : cap;
}

// Every per-frame kernel is launched with programmatic stream serialisation,
// so its prologue overlaps the previous kernel's tail (see waitPrevGrid).
template <class... Args>
static cudaError_t launchPdl(void (*kernel)(Args...), int grid, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

cudaError_t launchRemap(const Segment* segs, int nsegs, int total, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_remap, gridFor(total, 8), st, segs, nsegs, total);
}

cudaError_t launchPyrDown(const Segment* segs, int nsegs, int total, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_pyrdown, gridFor(total, 6), st, segs, nsegs, total);
}

cudaError_t launchBlend(const Segment* segs, int nsegs, int total, cudaStream_t st)
{
    if (total <= 0) return cudaSuccess;
    return launchPdl(k_blend, gridFor(total, 8), st, segs, nsegs, total);
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
