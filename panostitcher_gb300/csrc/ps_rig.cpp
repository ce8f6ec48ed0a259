// ps_rig.cpp -- prepare-time construction of a rig's resident state and the
// launch plans that stitch frames with it.
#include "ps_rig.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdarg>
#include <cstdio>

namespace ps {

static std::atomic<uint64_t> g_generation{1};

// Largest Gaussian radius of the linear-blend weights (2r+1 taps per pass).
constexpr int kMaxLinearRadius = 1024;

// Fixed-point taps of a (2r+1)-tap Gaussian with sigma r/3: the kernel of
// cv::getGaussianKernel(2r+1, r/3, CV_32F) (exp in double, each term and
// the normalised term stored as float) scaled by 2^8 and rounded to the
// nearest integer, ties to even.
static std::vector<int> gaussTaps(int r)
{
    const int n = 2 * r + 1;
    const double sigma = r / 3.0;  // source/Blend/LinearBlend.cpp:142
    const double scale2X = -0.5 / (sigma * sigma);
    std::vector<float> f(n);
    double sum = 0;
    for (int i = 0; i < n; i++) {
        const double x = i - (n - 1) * 0.5;
        f[i] = (float)std::exp(scale2X * x * x);
        sum += f[i];
    }
    sum = 1. / sum;
    std::vector<int> q(n);
    for (int i = 0; i < n; i++) {
        const float k = (float)(f[i] * sum);
        q[i] = (int)std::nearbyint((double)k * 256.0);
    }
    return q;
}

[[noreturn]] void fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error(code, buf);
}

void checkCuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    cudaGetLastError();  // clear a non-sticky error
    fail(e == cudaErrorMemoryAllocation ? PS_ENOMEM : PS_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ---- buffers ---------------------------------------------------------------------
void DevBuf::alloc(size_t bytes)
{
    reset();
    if (!bytes) return;
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(PS_ENOMEM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
    p_ = p;
    n_ = bytes;
}

void DevBuf::reset()
{
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
}

void DevBuf::zero(cudaStream_t st)
{
    if (p_) PS_CUDA(cudaMemsetAsync(p_, 0, n_, st));
}

void HostBuf::alloc(size_t bytes)
{
    reset();
    if (!bytes) return;
    void* p = nullptr;
    const cudaError_t e = cudaMallocHost(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(PS_ENOMEM, "pinned allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
    p_ = p;
    n_ = bytes;
}

void HostBuf::reset()
{
    if (p_) cudaFreeHost(p_);
    p_ = nullptr;
    n_ = 0;
}

static inline int divUp(int a, int b) { return (a + b - 1) / b; }
static inline int roundUp(int a, int b) { return divUp(a, b) * b; }

// ---- Rig ---------------------------------------------------------------------------
void Rig::clear()
{
    waitIdleQuiet();  // kernels and downloads of earlier frames may still use the buffers
    for (auto& l : lv_) {
        for (int k = 0; k < kIoSlots; k++) {
            l.G[k].reset();
            l.C[k].reset();
        }
        l.Wt.reset();
        l.Am.reset();
    }
    nextSlot_ = lastSlot_ = 0;
    maps_.reset(); union_.reset(); inputs_.reset(); output_.reset(); covDev_.reset(); status_.reset(); planar_.reset();
    camsF_.reset(); covTiles_.reset();
    imgArgs_.reset(); dDesc_.reset(); dRemap_.reset(); dDown_.reset(); dBlend_.reset(); dCams_.reset();
    tmaps_.reset();
    hRemap_.clear();
    hDown_.clear();
    hBlend_.clear();
    hCams_.clear();
    tailDown_ = tailBlend_ = 1;
    for (int j = 0; j <= PS_MAX_LEVELS; j++) downOff_[j] = downCnt_[j] = blendOff_[j] = blendCnt_[j] = 0;
    covCount_ = weightCount_ = alphaCount_ = 0;
    covBits_.clear();
    seamBits_.clear();
    geom_.clear();
    n_ = W_ = H_ = L_ = full_ = srcW_ = srcH_ = 0;
    hasMaps_ = linear_ = custom_ = false;
    numLinear_ = 0;
    dLinear_.reset();
    linW_.reset();
    inPitch_ = 0;
    gen_ = 0;
}

Rig::~Rig()
{
    waitIdleQuiet();
    for (cudaEvent_t* es : {slotComputed_, slotDownloaded_})
        for (int k = 0; k < kIoSlots; k++)
            if (es[k]) cudaEventDestroy(es[k]);
}

cudaEvent_t Rig::slotEvent(cudaEvent_t& e)
{
    if (!e) PS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return e;
}

void Rig::setGeometry(int n, int W, int H, int L)
{
    slots_ = slotsWanted_;
    nextSlot_ = lastSlot_ = 0;
    n_ = n;
    W_ = W;
    H_ = H;
    L_ = L;
    geom_.resize(L + 1);
    int w = W, h = H;
    for (int j = 0; j <= L; j++) {
        geom_[j] = {w, h, roundUp(w, 64)};
        w = (w + 1) / 2;  // getPyramidLevelSizes, source/CudaAccel/CudaMultibandBlend.cpp:486-492
        h = (h + 1) / 2;
    }
}

long long Rig::residentBytes() const
{
    long long b = 0;
    for (const auto& l : lv_) {
        for (int k = 0; k < kIoSlots; k++) b += l.G[k].bytes() + l.C[k].bytes();
        b += l.Wt.bytes() + l.Am.bytes();
    }
    b += maps_.bytes() + union_.bytes() + inputs_.bytes() + output_.bytes() + covDev_.bytes() + status_.bytes();
    b += imgArgs_.bytes() + dDesc_.bytes() + dRemap_.bytes() + dDown_.bytes() + dBlend_.bytes() + dCams_.bytes();
    b += tmaps_.bytes();
    b += dLinear_.bytes() + linW_.bytes() + planar_.bytes() + camsF_.bytes() + covTiles_.bytes();
    return b;
}

static void validateParams(const ps_photo_param* params, int n, int srcW, int srcH, int dstW, int dstH)
{
    if (!params || n <= 0) fail(PS_EINVAL, "no camera parameters");
    if (n > PS_MAX_CAMS) fail(PS_EINVAL, "%d cameras, at most %d supported", n, PS_MAX_CAMS);
    // source/Task/RicohUtil.cpp:1098-1103
    if (!((dstW & 1) == 0 && (dstH & 1) == 0 && dstH * 2 == dstW) || dstW <= 0)
        fail(PS_EINVAL, "dstSize (%d, %d) not qualified: width and height must be even and width == 2 * height",
             dstW, dstH);
    if (srcW <= 0 || srcH <= 0) fail(PS_EINVAL, "srcSize (%d, %d) must be positive", srcW, srcH);
    for (int i = 0; i < n; i++)
        if (params[i].image_type < 0 || params[i].image_type > 3)
            fail(PS_EINVAL, "camera %d: image_type %d not in 0..3", i, params[i].image_type);
}

// Upper bound of the work lists and descriptors a rig of this shape holds:
// every pyrDown and blend tile listed (with its camera list), remap items for
// every camera's level-0 tiles, one descriptor and one set of tensor maps per
// state slot.
static long long listBytes(int W, int H, int n, int L, int slots)
{
    long long b = (long long)(sizeof(RigDev) + (size_t)(L + 1) * kTmapsPerLevel * sizeof(CUtensorMap)) * slots + 4096;
    int w = W, h = H;
    for (int j = 0; j <= L; j++) {
        const long long down = (long long)divUp(w, kDownTW) * divUp(h, kDownTH) * n;
        const long long blend = (long long)divUp(w, kBlendTW) * divUp(h, kBlendTH);
        b += (j ? down * (long long)sizeof(DownItem) : 0) + blend * ((long long)sizeof(BlendItem) + n);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    // remap items and each state slot's tie list
    return b + (long long)divUp(W, kRemapTW) * divUp(H, kRemapTH) * n *
                   (sizeof(RemapItem) + sizeof(RemapTie) * kRemapTiesPerTile * slots);
}

long long Rig::estimateBlenderBytes(int W, int H, int n, int maxLevels, int slots)
{
    if (W <= 0 || H <= 0 || n <= 0 || n > PS_MAX_CAMS) fail(PS_EINVAL, "size (%d, %d) or %d images invalid", W, H, n);
    if (slots < 1 || slots > kIoSlots) fail(PS_EINVAL, "%d state slots, 1..%d supported", slots, kIoSlots);
    const int L = std::max(0, trueNumLevels(W, H, maxLevels, 2));
    long long b = 0;
    int w = W, h = H;
    for (int j = 0; j <= L; j++) {
        const long long px = (long long)roundUp(w, 64) * h;
        b += px * n * (4 * slots + 2 + (j ? 2 : 0)) + (j ? px * 8 * slots : 0);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    // coverage masks (input checks), union mask, output staging, input arguments, lists
    return b + (long long)W * H * n + (long long)roundUp(W, 64) * H + (long long)W * H * 4 * slots + 16LL * n +
           listBytes(W, H, n, L, slots);
}

long long Rig::estimateBytes(const ps_photo_param* params, int n, int blendParam, int srcW, int srcH, int dstW,
                             int dstH, int slots, bool mapFree)
{
    validateParams(params, n, srcW, srcH, dstW, dstH);
    const int L = std::max(0, trueNumLevels(dstW, dstH, blendParam, 2));
    long long b = 0;
    int w = dstW, h = dstH;
    for (int j = 0; j <= L; j++) {
        const long long px = (long long)roundUp(w, 64) * h;
        b += px * n * (4 * slots + 2 + (j ? 2 : 0)) + (j ? px * 8 * slots : 0);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    // maps (or, map-free, coverage bits) bounded by the full canvas per
    // camera, inputs, output, union mask, lists
    const long long tiles = (long long)divUp(dstW, kRemapTW) * divUp(dstH, kRemapTH) * n;
    b += (mapFree ? tiles * kRemapTH * 4 + (long long)sizeof(RemapParamF) * n : (long long)dstW * dstH * 8 * n) +
         ((long long)roundUp(srcW * 4, 256) * srcH * n + (long long)dstW * dstH * 4) * slots +
         (long long)roundUp(dstW, 64) * dstH + listBytes(dstW, dstH, n, L, slots);
    return b;
}

// getNonIntersectingMasks of n device coverage masks into seam (device).
static void distanceSeams(const uint8_t* cov, int n, int W, int H, uint8_t* seam, cudaStream_t st)
{
    const size_t npx = (size_t)W * H;
    DevBuf uni(npx), dUni(npx * 4), dCam(npx * 4);
    PS_CUDA(launchNonIntersectingMasks(cov, n, W, H, seam, uni.as<uint8_t>(), dUni.as<int32_t>(), dCam.as<int32_t>(),
                                       st));
    PS_CUDA(cudaStreamSynchronize(st));  // before the scratch is freed
}

// Explicit seam masks must not intersect, as getNonIntersectingMasks'
// never do (source/Blend/Mask.cpp:376-398): the collapsed levels are int16,
// which holds only while the seam weights at a pixel sum to at most 256 at
// level 0 (and 256 + n*j/2 at level j, from the per-level rounding).
static void checkSeamsDisjoint(const uint8_t* const* seams, int n, int W, int H)
{
    const size_t npx = (size_t)W * H;
    // branch-free count of the seams holding each pixel (n <= 64 fits a byte)
    std::vector<uint8_t> count(npx, 0);
    for (int i = 0; i < n; i++) {
        const uint8_t* s = seams[i];
        uint8_t* c = count.data();
        for (size_t p = 0; p < npx; p++) c[p] = (uint8_t)(c[p] + (s[p] != 0));
    }
    uint8_t most = 0;
    for (size_t p = 0; p < npx; p++) most = std::max(most, count[p]);
    if (most <= 1) return;
    // a shared pixel: name the first one, in camera order
    std::vector<uint8_t> owner(npx, 0);  // 1 + the camera whose seam holds the pixel
    for (int i = 0; i < n; i++) {
        const uint8_t* s = seams[i];
        for (size_t p = 0; p < npx; p++) {
            if (!s[p]) continue;
            if (owner[p])
                fail(PS_EINVAL, "seam masks %d and %d intersect at (%d, %d)", owner[p] - 1, i, (int)(p % W),
                     (int)(p / W));
            owner[p] = (uint8_t)(i + 1);
        }
    }
}

void Rig::prepareFromParams(const ps_photo_param* params, int n, int blendParam, int srcW, int srcH, int dstW,
                            int dstH, const uint8_t* const* seams, cudaStream_t st, int seamRule, int highQuality)
{
    NvtxRange range("ps.prepare");
    clear();
    validateParams(params, n, srcW, srcH, dstW, dstH);
    if (blendParam <= 0) fail(PS_EINVAL, "blendParam = %d, should be positive", blendParam);  // RicohUtil.cpp:1105
    if (!highQuality && blendParam > kMaxLinearRadius)
        fail(PS_EINVAL, "blendParam = %d, the linear-blend radius is at most %d", blendParam, kMaxLinearRadius);
    if (seams) {
        for (int i = 0; i < n; i++)
            if (!seams[i]) fail(PS_EINVAL, "seam mask %d is NULL", i);
        checkSeamsDisjoint(seams, n, dstW, dstH);
    }
    // The reference compares its estimate of the stream-based render's
    // device memory with the free memory and, within 500 MB, falls back to
    // one camera at a time (source/Task/RicohUtil.cpp:1135-1170).  Here the
    // resident state is per frame in flight, so the fallback is fewer state
    // slots: as many as fit with that margin, down to one.
    // A caller's memory budget (setMemoryBudget) caps the same estimate.
    // When even one slot does not fit, the maps stop being resident: the
    // remap computes each source coordinate (the reference's map-free
    // remap, RicohUtil.cpp:1315-1329).
    int slots = slotsWanted_;
    mapFree_ = highQuality && mapFreeWanted_;
    if (highQuality) {
        size_t freeB = 0, totalB = 0;
        PS_CUDA(cudaMemGetInfo(&freeB, &totalB));
        long long room = (long long)freeB - 500000000LL;
        if (budget_ > 0) room = std::min(room, budget_);
        while (slots > 1 && estimateBytes(params, n, blendParam, srcW, srcH, dstW, dstH, slots, mapFree_) > room)
            slots--;
        if (!mapFree_ && estimateBytes(params, n, blendParam, srcW, srcH, dstW, dstH, slots, false) > room)
            mapFree_ = true;
    }
    try {
        // MIN_SIDE_LENGTH = 2, source/Task/RicohUtil.cpp:15
        setGeometry(n, dstW, dstH, highQuality ? std::max(0, trueNumLevels(dstW, dstH, blendParam, 2)) : 0);
        lowMemory_ = slots < slots_ || (mapFree_ && !mapFreeWanted_);
        slots_ = slots;
        srcW_ = srcW;
        srcH_ = srcH;
        const size_t npx = (size_t)dstW * dstH;
        DevBuf xmap(n * npx * 4), ymap(n * npx * 4), cov(n * npx), seam(n * npx);
        std::vector<RemapDev>& rp = hParams_;
        rp.assign(n, RemapDev{});
        for (int i = 0; i < n; i++) remapInit(params[i], dstW, dstH, srcW, srcH, rp[i]);
        DevBuf dParams(sizeof(RemapDev) * n);
        PS_CUDA(cudaMemcpyAsync(dParams.get(), rp.data(), sizeof(RemapDev) * n, cudaMemcpyHostToDevice, st));
        for (int i = 0; i < n; i++)
            PS_CUDA(launchGenMap(dParams.as<RemapDev>() + i, dstW, dstH, xmap.as<float>() + i * npx,
                                 ymap.as<float>() + i * npx, cov.as<uint8_t>() + i * npx, st));
        if (seams) {
            for (int i = 0; i < n; i++)
                PS_CUDA(cudaMemcpyAsync(seam.as<uint8_t>() + i * npx, seams[i], npx, cudaMemcpyHostToDevice, st));
        } else if (seamRule == PS_SEAMS_DISTANCE) {
            distanceSeams(cov.as<uint8_t>(), n, dstW, dstH, seam.as<uint8_t>(), st);
        } else {
            PS_CUDA(launchNearestAxisSeams(dParams.as<RemapDev>(), n, dstW, dstH, cov.as<uint8_t>(),
                                           seam.as<uint8_t>(), st));
        }
        hasMaps_ = true;
        inPitch_ = roundUp(srcW * 4, 256);
        inputs_.alloc((size_t)inPitch_ * srcH * n * slots_);
        inputs_.zero(st);
        output_.alloc(npx * 4 * slots_);
        if (highQuality) preparePyramids(cov.as<uint8_t>(), seam.as<uint8_t>(), xmap.as<float>(), ymap.as<float>(), st);
        else prepareLinear(cov.as<uint8_t>(), seam.as<uint8_t>(), xmap.as<float>(), ymap.as<float>(), blendParam, st);
        PS_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        clear();
        throw;
    }
}

void Rig::prepareFromMasks(const uint8_t* const* masks, const uint8_t* const* seams, int n, int W, int H,
                           int maxLevels, int minLength, cudaStream_t st)
{
    NvtxRange range("ps.prepare");
    clear();
    // CudaTilingMultibandBlendFast::prepare, source/CudaAccel/CudaMultibandBlend.cpp:549-568
    if (!masks || n <= 0) fail(PS_EINVAL, "no masks");
    if (n > PS_MAX_CAMS) fail(PS_EINVAL, "%d masks, at most %d supported", n, PS_MAX_CAMS);
    if (W <= 0 || H <= 0) fail(PS_EINVAL, "mask size (%d, %d) must be positive", W, H);
    for (int i = 0; i < n; i++)
        if (!masks[i] || (seams && !seams[i])) fail(PS_EINVAL, "mask %d is NULL", i);
    if (seams) checkSeamsDisjoint(seams, n, W, H);
    try {
        setGeometry(n, W, H, std::max(0, trueNumLevels(W, H, maxLevels, minLength)));
        const size_t npx = (size_t)W * H;
        covDev_.alloc(n * npx);
        DevBuf seam(n * npx);
        for (int i = 0; i < n; i++) {
            PS_CUDA(cudaMemcpyAsync(covDev_.as<uint8_t>() + i * npx, masks[i], npx, cudaMemcpyHostToDevice, st));
            if (seams)
                PS_CUDA(cudaMemcpyAsync(seam.as<uint8_t>() + i * npx, seams[i], npx, cudaMemcpyHostToDevice, st));
        }
        // CudaMultibandBlend.cpp:570-571
        if (!seams) distanceSeams(covDev_.as<uint8_t>(), n, W, H, seam.as<uint8_t>(), st);
        output_.alloc(npx * 4 * slots_);
        imgArgs_.alloc((sizeof(void*) + sizeof(long long)) * n);
        preparePyramids(covDev_.as<uint8_t>(), seam.as<uint8_t>(), nullptr, nullptr, st);
        PS_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        clear();
        throw;
    }
}

static void packBits(const std::vector<uint8_t>& in, std::vector<uint8_t>& out)
{
    out.assign((in.size() + 7) / 8, 0);
    for (size_t i = 0; i < in.size(); i++)
        if (in[i]) out[i >> 3] |= (uint8_t)(1u << (i & 7));
}

void Rig::preparePyramids(const uint8_t* cov, const uint8_t* seam, const float* xmap, const float* ymap,
                          cudaStream_t st)
{
    const int n = n_, L = L_, W = W_, H = H_;
    const size_t npx = (size_t)W * H;
    // resident pyramids (zeroed: tiles outside a camera's support stay 0)
    for (int j = 0; j <= L; j++) {
        const LevelGeom& g = geom_[j];
        const size_t plane = (size_t)g.pitch * g.h;
        for (int k = 0; k < slots_; k++) {
            lv_[j].G[k].alloc(plane * n * 4);
            lv_[j].G[k].zero(st);
        }
        lv_[j].Wt.alloc(plane * n * 2);
        lv_[j].Wt.zero(st);
        if (j > 0) {
            lv_[j].Am.alloc(plane * n * 2);
            lv_[j].Am.zero(st);
            for (int k = 0; k < slots_; k++) {
                lv_[j].C[k].alloc(plane * 8);
                lv_[j].C[k].zero(st);
            }
        }
    }
    union_.alloc((size_t)geom_[0].pitch * H);
    union_.zero(st);
    status_.alloc(sizeof(int));
    status_.zero(st);

    // weight and alpha pyramids (CudaMultibandBlend.cpp:586-605)
    {
        const size_t plane0 = (size_t)geom_[0].pitch * H;
        DevBuf a0(plane0 * n * 2), a1(plane0 * n * 2);
        a0.zero(st);
        a1.zero(st);
        PS_CUDA(launchInitLevel0(cov, seam, W, H, (long long)npx, lv_[0].Wt.as<uint16_t>(), a0.as<uint16_t>(),
                                 geom_[0].pitch, (long long)plane0, n, st));
        uint16_t* cur = a0.as<uint16_t>();
        uint16_t* nxt = a1.as<uint16_t>();
        for (int j = 0; j < L; j++) {
            const LevelGeom& s = geom_[j];
            const LevelGeom& d = geom_[j + 1];
            const long long ss = (long long)s.pitch * s.h, ds = (long long)d.pitch * d.h;
            PS_CUDA(launchAlphaDown(cur, s.w, s.h, s.pitch, ss, lv_[j + 1].Am.as<uint16_t>(), nxt, d.w, d.h, d.pitch,
                                    ds, n, st));
            PS_CUDA(launchWeightDown(lv_[j].Wt.as<uint16_t>(), s.w, s.h, s.pitch, ss, lv_[j + 1].Wt.as<uint16_t>(),
                                     d.w, d.h, d.pitch, ds, n, st));
            std::swap(cur, nxt);
        }
        PS_CUDA(cudaStreamSynchronize(st));
    }

    // tile activity flags of the remap and the pyrDown levels
    const int rX = divUp(W, kRemapTW), rY = divUp(H, kRemapTH);
    DevBuf rflags((size_t)n * rX * rY);
    if (xmap) {
        rflags.zero(st);
        PS_CUDA(launchTileFlags8(cov, W, H, W, (long long)npx, n, kRemapTW, kRemapTH, rX, rY, rflags.as<uint8_t>(), st));
    }
    std::vector<DevBuf> dflags(L + 1);
    DevBuf counts(sizeof(unsigned long long));
    counts.zero(st);
    for (int j = 1; j <= L; j++) {
        const LevelGeom& g = geom_[j];
        const long long stride = (long long)g.pitch * g.h;
        const int dX = divUp(g.w, kDownTW), dY = divUp(g.h, kDownTH);
        dflags[j].alloc((size_t)n * dX * dY);
        dflags[j].zero(st);
        PS_CUDA(launchTileFlags16(lv_[j].Am.as<uint16_t>(), g.w, g.h, g.pitch, stride, n, kDownTW, kDownTH, dX, dY,
                                  dflags[j].as<uint8_t>(), st));
        PS_CUDA(launchCountNonzero16(lv_[j].Am.as<uint16_t>(), g.w, g.h, g.pitch, stride, n,
                                     counts.as<unsigned long long>(), st));
    }
    unsigned long long hAlpha = 0;
    std::vector<uint8_t> hR(xmap ? rflags.bytes() : 0);
    std::vector<std::vector<uint8_t>> hD(L + 1);
    PS_CUDA(cudaMemcpyAsync(&hAlpha, counts.get(), sizeof hAlpha, cudaMemcpyDeviceToHost, st));
    if (xmap) PS_CUDA(cudaMemcpyAsync(hR.data(), rflags.get(), hR.size(), cudaMemcpyDeviceToHost, st));
    for (int j = 1; j <= L; j++) {
        hD[j].resize(dflags[j].bytes());
        PS_CUDA(cudaMemcpyAsync(hD[j].data(), dflags[j].get(), hD[j].size(), cudaMemcpyDeviceToHost, st));
    }
    std::vector<uint8_t> hCov(n * npx), hSeam(n * npx);
    PS_CUDA(cudaMemcpyAsync(hCov.data(), cov, n * npx, cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaMemcpyAsync(hSeam.data(), seam, n * npx, cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaStreamSynchronize(st));
    alphaCount_ = (long long)hAlpha;
    covCount_ = 0;
    for (uint8_t v : hCov) covCount_ += v != 0;
    packBits(hCov, covBits_);
    packBits(hSeam, seamBits_);
    hCov.clear();
    hSeam.clear();

    // work items of the remap and the pyrDown levels
    hRemap_.clear();
    if (xmap) {
        uint32_t t = 0;
        for (int c = 0; c < n; c++)
            for (int ty = 0; ty < rY; ty++)
                for (int tx = 0; tx < rX; tx++)
                    if (hR[((size_t)c * rY + ty) * rX + tx])
                        hRemap_.push_back({(uint16_t)c, 0, (uint16_t)tx, (uint16_t)ty, t++});
    }
    std::vector<DownItem> down;
    for (int j = 1; j <= L; j++) {
        const int dX = divUp(geom_[j].w, kDownTW), dY = divUp(geom_[j].h, kDownTH);
        downOff_[j] = (int)down.size();
        for (int c = 0; c < n; c++)
            for (int ty = 0; ty < dY; ty++)
                for (int tx = 0; tx < dX; tx++)
                    if (hD[j][((size_t)c * dY + ty) * dX + tx])
                        down.push_back({(uint8_t)c, (uint8_t)j, (uint16_t)tx, (uint16_t)ty, 0});
        downCnt_[j] = (int)down.size() - downOff_[j];
    }
    hDown_ = down;
    // the weights' part: union coverage, fullMask, blend items
    buildBlendState(cov, false, st);
    // levels with few tiles (from the top down) go to the tail kernel
    tailSplit(shape_.tailMaxItems, &tailDown_, &tailBlend_);
    dRemap_.alloc(std::max<size_t>(1, hRemap_.size()) * sizeof(RemapItem));
    dDown_.alloc(std::max<size_t>(1, down.size()) * sizeof(DownItem));
    if (!hRemap_.empty())
        PS_CUDA(cudaMemcpyAsync(dRemap_.get(), hRemap_.data(), hRemap_.size() * sizeof(RemapItem),
                                cudaMemcpyHostToDevice, st));
    if (!down.empty())
        PS_CUDA(cudaMemcpyAsync(dDown_.get(), down.data(), down.size() * sizeof(DownItem), cudaMemcpyHostToDevice, st));

    // tile-compact maps of the covered remap tiles
    if (xmap && !hRemap_.empty() && !mapFree_) {
        maps_.alloc(hRemap_.size() * kRemapTW * kRemapTH * sizeof(float2));
        PS_CUDA(launchCompactMaps(xmap, ymap, W, H, (long long)npx, dRemap_.as<RemapItem>(), (int)hRemap_.size(),
                                  maps_.as<float2>(), st));
    }
    if (xmap && !hRemap_.empty() && mapFree_) {  // coverage bits and fp32 parameters instead of maps
        covTiles_.alloc(hRemap_.size() * kRemapTH * sizeof(uint32_t));
        PS_CUDA(launchCovTiles(cov, W, H, (long long)npx, dRemap_.as<RemapItem>(), (int)hRemap_.size(),
                               covTiles_.as<uint32_t>(), st));
        std::vector<RemapParamF> pf(n);
        for (int i = 0; i < n; i++) pf[i] = remapParamF(hParams_[i]);
        camsF_.alloc(sizeof(RemapParamF) * n);
        PS_CUDA(cudaMemcpyAsync(camsF_.get(), pf.data(), sizeof(RemapParamF) * n, cudaMemcpyHostToDevice, st));
        PS_CUDA(cudaStreamSynchronize(st));  // pf is a host temporary
    }

    // device descriptor
    RigDev d;
    std::memset(&d, 0, sizeof d);
    d.n = n;
    d.L = L;
    d.W = W;
    d.H = H;
    d.full = full_;
    d.srcW = srcW_;
    d.srcH = srcH_;
    d.maps = mapFree_ ? nullptr : maps_.as<float2>();
    d.numRemapItems = (int)hRemap_.size();
    d.camsF = camsF_.as<RemapParamF>();
    d.covTiles = covTiles_.as<uint32_t>();
    d.unionMask = union_.as<uint8_t>();
    d.camLists = dCams_.as<uint8_t>();
    d.downItems = dDown_.as<DownItem>();
    d.blendItems = dBlend_.as<BlendItem>();
    for (int j = 0; j <= L; j++) {
        d.downOff[j] = downOff_[j];
        d.downCnt[j] = downCnt_[j];
        d.blendOff[j] = blendOff_[j];
        d.blendCnt[j] = blendCnt_[j];
    }
    d.tailDown = tailDown_;
    d.tailBlend = tailBlend_;
    d.tailHalf = shape_.tailHalf;
    for (int j = 0; j <= L; j++) {
        const LevelGeom& g = geom_[j];
        d.lv[j].w = g.w;
        d.lv[j].h = g.h;
        d.lv[j].pitch = g.pitch;
        d.lv[j].camStride = (long long)g.pitch * g.h;
        d.lv[j].Wt = lv_[j].Wt.as<uint16_t>();
        d.lv[j].Am = lv_[j].Am.as<uint16_t>();
    }
    hDesc_ = d;
    dDesc_.alloc(sizeof(RigDev) * slots_);
    writeDescriptors(st);
    gen_ = g_generation++;
}

static void unpackBits(const std::vector<uint8_t>& bits, size_t count, std::vector<uint8_t>& out)
{
    out.resize(count);
    for (size_t i = 0; i < count; i++) out[i] = (bits[i >> 3] >> (i & 7)) & 1 ? 255 : 0;
}

// The state that follows the weights: the union mask and the fullMask flag
// from uniSrc (n device masks: the coverage, or the custom masks, whose
// blend always normalises by the weight sums), the level-0 tile classes,
// the count of non-zero weights and the blend items of every level
// (CudaMultibandBlend.cpp:606-642; with custom masks :838-860, 888-892).
void Rig::buildBlendState(const uint8_t* uniSrc, bool custom, cudaStream_t st)
{
    const int n = n_, L = L_, W = W_, H = H_;
    const size_t npx = (size_t)W * H;
    const int bX0 = divUp(W, kBlendTW), bY0 = divUp(H, kBlendTH);
    DevBuf tileCounts((size_t)bX0 * bY0 * sizeof(int)), total(sizeof(unsigned long long));
    total.zero(st);
    PS_CUDA(launchUnion(uniSrc, n, W, H, (long long)npx, union_.as<uint8_t>(), geom_[0].pitch, kBlendTW, kBlendTH, bX0,
                        tileCounts.as<int>(), total.as<unsigned long long>(), st));
    std::vector<DevBuf> bflags(L + 1), uflags(L + 1);
    DevBuf counts(sizeof(unsigned long long));
    counts.zero(st);
    for (int j = 0; j <= L; j++) {
        const LevelGeom& g = geom_[j];
        const long long stride = (long long)g.pitch * g.h;
        const int bX = divUp(g.w, kBlendTW), bY = divUp(g.h, kBlendTH);
        bflags[j].alloc((size_t)n * bX * bY);
        bflags[j].zero(st);
        uflags[j].alloc((size_t)n * bX * bY);
        uflags[j].zero(st);
        PS_CUDA(launchTileNot256(lv_[j].Wt.as<uint16_t>(), g.w, g.h, g.pitch, stride, n, kBlendTW, kBlendTH, bX, bY,
                                 uflags[j].as<uint8_t>(), st));
        PS_CUDA(launchTileFlags16(lv_[j].Wt.as<uint16_t>(), g.w, g.h, g.pitch, stride, n, kBlendTW, kBlendTH, bX, bY,
                                  bflags[j].as<uint8_t>(), st));
        PS_CUDA(launchCountNonzero16(lv_[j].Wt.as<uint16_t>(), g.w, g.h, g.pitch, stride, n,
                                     counts.as<unsigned long long>(), st));
    }
    std::vector<int> hCounts((size_t)bX0 * bY0);
    unsigned long long hTotal = 0, hWeights = 0;
    std::vector<std::vector<uint8_t>> hB(L + 1), hU(L + 1);
    PS_CUDA(cudaMemcpyAsync(hCounts.data(), tileCounts.get(), tileCounts.bytes(), cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaMemcpyAsync(&hTotal, total.get(), sizeof hTotal, cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaMemcpyAsync(&hWeights, counts.get(), sizeof hWeights, cudaMemcpyDeviceToHost, st));
    for (int j = 0; j <= L; j++) {
        hB[j].resize(bflags[j].bytes());
        PS_CUDA(cudaMemcpyAsync(hB[j].data(), bflags[j].get(), hB[j].size(), cudaMemcpyDeviceToHost, st));
        hU[j].resize(uflags[j].bytes());
        PS_CUDA(cudaMemcpyAsync(hU[j].data(), uflags[j].get(), hU[j].size(), cudaMemcpyDeviceToHost, st));
    }
    PS_CUDA(cudaStreamSynchronize(st));
    full_ = !custom && hTotal == (unsigned long long)npx;  // CudaMultibandBlend.cpp:616-617
    weightCount_ = (long long)hWeights;

    std::vector<BlendItem> blend;
    std::vector<uint8_t> cams;
    for (int j = 0; j <= L; j++) {
        const LevelGeom& g = geom_[j];
        const int bX = divUp(g.w, kBlendTW), bY = divUp(g.h, kBlendTH);
        blendOff_[j] = (int)blend.size();
        for (int ty = 0; ty < bY; ty++)
            for (int tx = 0; tx < bX; tx++) {
                std::vector<uint8_t> list;
                for (int c = 0; c < n; c++)
                    if (hB[j][((size_t)c * bY + ty) * bX + tx]) list.push_back((uint8_t)c);
                uint8_t cls = 0;
                if (j == 0) {
                    const int tw = std::min(kBlendTW, g.w - tx * kBlendTW), th = std::min(kBlendTH, g.h - ty * kBlendTH);
                    const int cnt = hCounts[(size_t)ty * bX0 + tx];
                    cls = cnt == 0 ? 0 : (cnt == tw * th ? 1 : 2);
                }
                BlendItem it;
                std::memset(&it, 0, sizeof it);
                it.level = (uint8_t)j;
                it.cls = cls;
                it.camCnt = (uint8_t)list.size();
                if (list.size() == 1 && !hU[j][((size_t)list[0] * bY + ty) * bX + tx]) it.flags |= kTileUniform;
                it.tx = (uint16_t)tx;
                it.ty = (uint16_t)ty;
                if (list.size() <= (size_t)kInlineCams) {
                    for (size_t q = 0; q < list.size(); q++) it.cams[q] = list[q];
                } else {
                    const uint32_t off = (uint32_t)cams.size();
                    std::memcpy(it.cams, &off, sizeof off);
                    cams.insert(cams.end(), list.begin(), list.end());
                }
                blend.push_back(it);
            }
        blendCnt_[j] = (int)blend.size() - blendOff_[j];
    }
    if (cams.empty()) cams.push_back(0);
    hBlend_ = blend;
    hCams_ = cams;
    dBlend_.alloc(std::max<size_t>(1, blend.size()) * sizeof(BlendItem));
    dCams_.alloc(cams.size());
    PS_CUDA(cudaMemcpyAsync(dBlend_.get(), blend.data(), blend.size() * sizeof(BlendItem), cudaMemcpyHostToDevice, st));
    PS_CUDA(cudaMemcpyAsync(dCams_.get(), cams.data(), cams.size(), cudaMemcpyHostToDevice, st));
}

void Rig::setCustomMasks(const uint8_t* const* masks, cudaStream_t st)
{
    if (!ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
    if (linear_) fail(PS_EINVAL, "custom masks need the multiband blend (highQualityBlend != 0)");
    if (masks)
        for (int i = 0; i < n_; i++)
            if (!masks[i]) fail(PS_EINVAL, "custom mask %d is NULL", i);
    // the descriptors and work lists change under no run
    waitIdle();
    const int n = n_, L = L_, W = W_, H = H_;
    const size_t npx = (size_t)W * H;
    // weight masks: the custom masks, or the prepared unique masks back
    DevBuf wm(n * npx), um;
    std::vector<uint8_t> host;
    if (masks) {
        for (int i = 0; i < n; i++)
            PS_CUDA(cudaMemcpyAsync(wm.as<uint8_t>() + i * npx, masks[i], npx, cudaMemcpyHostToDevice, st));
    } else {
        unpackBits(seamBits_, n * npx, host);
        PS_CUDA(cudaMemcpyAsync(wm.get(), host.data(), n * npx, cudaMemcpyHostToDevice, st));
        PS_CUDA(cudaStreamSynchronize(st));
        um.alloc(n * npx);
        unpackBits(covBits_, n * npx, host);
        PS_CUDA(cudaMemcpyAsync(um.get(), host.data(), n * npx, cudaMemcpyHostToDevice, st));
    }
    // weight pyramids (pyramidDown16SC1To16SC1 of the 0/256 masks, CudaMultibandBlend.cpp:845-854)
    {
        const size_t plane0 = (size_t)geom_[0].pitch * H;
        // the kernel also writes an alpha level 0 from its coverage input: given the same masks and the same
        // output, both writes store the same value
        PS_CUDA(launchInitLevel0(wm.as<uint8_t>(), wm.as<uint8_t>(), W, H, (long long)npx, lv_[0].Wt.as<uint16_t>(),
                                 lv_[0].Wt.as<uint16_t>(), geom_[0].pitch, (long long)plane0, n, st));
        for (int j = 0; j < L; j++) {
            const LevelGeom& sg = geom_[j];
            const LevelGeom& dg = geom_[j + 1];
            PS_CUDA(launchWeightDown(lv_[j].Wt.as<uint16_t>(), sg.w, sg.h, sg.pitch, (long long)sg.pitch * sg.h,
                                     lv_[j + 1].Wt.as<uint16_t>(), dg.w, dg.h, dg.pitch, (long long)dg.pitch * dg.h,
                                     n, st));
        }
    }
    buildBlendState(masks ? wm.as<uint8_t>() : um.as<uint8_t>(), masks != nullptr, st);
    custom_ = masks != nullptr;
    tailSplit(shape_.tailMaxItems, &tailDown_, &tailBlend_);
    hDesc_.full = full_;
    hDesc_.camLists = dCams_.as<uint8_t>();
    hDesc_.blendItems = dBlend_.as<BlendItem>();
    for (int j = 0; j <= L; j++) {
        hDesc_.blendOff[j] = blendOff_[j];
        hDesc_.blendCnt[j] = blendCnt_[j];
    }
    hDesc_.tailDown = tailDown_;
    hDesc_.tailBlend = tailBlend_;
    writeDescriptors(st);  // synchronises
    gen_ = g_generation++;
}

// The driver's tensor-map encoder, looked up once through the runtime.
static PFN_cuTensorMapEncodeTiled_v12000 tensorMapEncoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// The tensor maps of k_blend's producer for every state slot and level (see
// kTmG ... kTmW): G and W as pitch x h x cameras, C as pitch x h.  Boxes lie
// inside the level wherever the producer uses them (interior tiles); the
// maps still bound them, filling zeros outside.
bool Rig::encodeTensorMaps()
{
    tmaps_.reset();
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensorMapEncoder();
    if (!encode || linear_) return false;
    const int perSlot = (L_ + 1) * kTmapsPerLevel;
    std::vector<CUtensorMap> maps((size_t)slots_ * perSlot);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    auto tiled = [&](CUtensorMap* m, CUtensorMapDataType type, size_t esz, void* base, int rank, cuuint64_t w,
                     cuuint64_t h, cuuint64_t cams, cuuint32_t bw, cuuint32_t bh, long long pitch, long long camStride) {
        const cuuint64_t dims[3] = {w, h, cams};
        const cuuint64_t strides[2] = {(cuuint64_t)pitch * esz, (cuuint64_t)camStride * esz};
        const cuuint32_t box[3] = {bw, bh, 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        return encode(m, type, (cuuint32_t)rank, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    for (int k = 0; k < slots_; k++)
        for (int j = 0; j <= L_; j++) {
            const LevelGeom& g = geom_[j];
            const long long cs = (long long)g.pitch * g.h;
            CUtensorMap* m = maps.data() + (size_t)k * perSlot + (size_t)j * kTmapsPerLevel;
            bool ok = tiled(m + kTmG, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, lv_[j].G[k].get(), 3, g.pitch, g.h, n_,
                            kBlendTW, kBlendTH, g.pitch, cs) &&
                      tiled(m + kTmGfp, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, lv_[j].G[k].get(), 3, g.pitch, g.h, n_,
                            kBlendTW / 2 + 8, kBlendTH / 2 + 2, g.pitch, cs) &&
                      tiled(m + kTmW, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, lv_[j].Wt.get(), 3, g.pitch, g.h, n_,
                            kBlendTW, kBlendTH, g.pitch, cs);
            if (ok && j > 0)
                ok = tiled(m + kTmC, CU_TENSOR_MAP_DATA_TYPE_UINT64, 8, lv_[j].C[k].get(), 2, g.pitch, g.h, 1,
                           kBlendTW / 2 + 4, kBlendTH / 2 + 2, g.pitch, cs);
            if (!ok) return false;
        }
    tmaps_.alloc(maps.size() * sizeof(CUtensorMap));
    PS_CUDA(cudaMemcpy(tmaps_.get(), maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
    return true;
}

// One descriptor per state slot, differing in the pyramid pointers.
void Rig::writeDescriptors(cudaStream_t st)
{
    RigDev ds[kIoSlots];
    const bool tma = encodeTensorMaps();
    for (int k = 0; k < slots_; k++) {
        ds[k] = hDesc_;
        ds[k].tmaps = tma ? static_cast<const uint8_t*>(tmaps_.get()) +
                                (size_t)k * (L_ + 1) * kTmapsPerLevel * sizeof(CUtensorMap)
                          : nullptr;
        for (int j = 0; j <= L_; j++) {
            ds[k].lv[j].G = lv_[j].G[k].as<uchar4>();
            ds[k].lv[j].C = lv_[j].C[k].as<short4>();
        }
    }
    PS_CUDA(cudaMemcpyAsync(dDesc_.get(), ds, sizeof(RigDev) * slots_, cudaMemcpyHostToDevice, st));
    PS_CUDA(cudaStreamSynchronize(st));
}

void Rig::waitIdle()
{
    for (int k = 0; k < kIoSlots; k++) {
        if (slotComputed_[k]) PS_CUDA(cudaEventSynchronize(slotComputed_[k]));
        if (slotDownloaded_[k]) PS_CUDA(cudaEventSynchronize(slotDownloaded_[k]));
    }
}

int Rig::takeStatus()
{
    waitIdle();
    if (!status_.get()) return 0;
    int v = 0;
    PS_CUDA(cudaMemcpy(&v, status_.get(), sizeof(int), cudaMemcpyDeviceToHost));
    if (v) PS_CUDA(cudaMemset(status_.get(), 0, sizeof(int)));
    return v;
}

void Rig::setWaitProbe(int polls)
{
    if (polls < 0 || polls > (1 << 24)) fail(PS_EINVAL, "wait probe of %d polls out of range 0..2^24", polls);
    if (polls == probe_) return;
    waitIdle();
    probe_ = polls;
    gen_++;  // plans re-record their launches
}

void Rig::waitIdleQuiet() noexcept
{
    for (cudaEvent_t* es : {slotComputed_, slotDownloaded_})
        for (int k = 0; k < kIoSlots; k++)
            if (es[k] && cudaEventSynchronize(es[k]) != cudaSuccess) cudaGetLastError();
}

void Rig::tailSplit(int maxItems, int* down, int* blend) const
{
    int d = L_ + 1, b = L_ + 1;
    while (d > 1 && downCnt_[d - 1] <= maxItems) d--;
    while (b > 0 && blendCnt_[b - 1] <= maxItems) b--;
    *down = d;
    *blend = b;
}

void Rig::setShape(const LaunchShape& s)
{
    if (s.tailMaxItems < 0 || s.tailMaxItems > (1 << 24)) fail(PS_EINVAL, "tail_max_items %d out of range", s.tailMaxItems);
    if (s.tailCluster != 0 && s.tailCluster != 8 && s.tailCluster != 16)
        fail(PS_EINVAL, "tail_cluster must be 0, 8 or 16 (got %d)", s.tailCluster);
    if (s.tailHalf != 0 && s.tailHalf != 1) fail(PS_EINVAL, "tail_half_tiles must be 0 or 1 (got %d)", s.tailHalf);
    if (s.remapDefer != 0 && s.remapDefer != 1)
        fail(PS_EINVAL, "remap_defer_ties must be 0 or 1 (got %d)", s.remapDefer);
    if (s.smallBlendMaxItems < 0 || s.smallBlendMaxItems > (1 << 24))
        fail(PS_EINVAL, "small_blend_max_items %d out of range", s.smallBlendMaxItems);
    for (int k = 0; k < 3; k++)
        if (s.ctasPerSm[k] < 0 || s.ctasPerSm[k] > 64)
            fail(PS_EINVAL, "ctas_per_sm[%d] = %d out of range 0..64", k, s.ctasPerSm[k]);
    if (s == shape_) return;
    shape_ = s;
    if (!ready() || linear_) return;
    // the descriptors change under no run: launch lists follow the new
    // generation (plans rebind), and no kernel may read the old split
    waitIdle();
    tailSplit(shape_.tailMaxItems, &tailDown_, &tailBlend_);
    hDesc_.tailDown = tailDown_;
    hDesc_.tailBlend = tailBlend_;
    hDesc_.tailHalf = shape_.tailHalf;
    writeDescriptors(nullptr);
    gen_ = g_generation++;
}

void Rig::prepareLinear(const uint8_t* cov, const uint8_t* seam, const float* xmap, const float* ymap, int radius,
                        cudaStream_t st)
{
    const int n = n_, W = W_, H = H_;
    const size_t npx = (size_t)W * H;
    linear_ = true;
    status_.alloc(sizeof(int));
    status_.zero(st);
    // the 32x16 tiles each camera covers
    const int rX = divUp(W, kRemapTW), rY = divUp(H, kRemapTH);
    DevBuf rflags((size_t)n * rX * rY);
    rflags.zero(st);
    PS_CUDA(launchTileFlags8(cov, W, H, W, (long long)npx, n, kRemapTW, kRemapTH, rX, rY, rflags.as<uint8_t>(), st));
    std::vector<uint8_t> hR(rflags.bytes()), hCov(n * npx), hSeam(n * npx);
    PS_CUDA(cudaMemcpyAsync(hR.data(), rflags.get(), hR.size(), cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaMemcpyAsync(hCov.data(), cov, n * npx, cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaMemcpyAsync(hSeam.data(), seam, n * npx, cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaStreamSynchronize(st));
    covCount_ = 0;
    std::vector<uint8_t> any(npx, 0);
    for (size_t c = 0; c < (size_t)n; c++)
        for (size_t p = 0; p < npx; p++)
            if (hCov[c * npx + p]) {
                covCount_++;
                any[p] = 1;
            }
    full_ = std::all_of(any.begin(), any.end(), [](uint8_t v) { return v != 0; });
    packBits(hCov, covBits_);
    packBits(hSeam, seamBits_);

    // work items: every canvas tile, with the covering cameras' remap items (index order)
    hRemap_.clear();
    std::vector<LinearItem> lin;
    lin.reserve((size_t)rX * rY);
    uint32_t t = 0;
    for (int ty = 0; ty < rY; ty++)
        for (int tx = 0; tx < rX; tx++) {
            const uint32_t first = (uint32_t)hRemap_.size();
            for (int c = 0; c < n; c++)
                if (hR[((size_t)c * rY + ty) * rX + tx]) hRemap_.push_back({(uint16_t)c, 0, (uint16_t)tx, (uint16_t)ty, t++});
            lin.push_back({(uint16_t)tx, (uint16_t)ty, first, (uint32_t)hRemap_.size() - first});
        }
    numLinear_ = (int)lin.size();
    dRemap_.alloc(std::max<size_t>(1, hRemap_.size()) * sizeof(RemapItem));
    dLinear_.alloc(lin.size() * sizeof(LinearItem));
    if (!hRemap_.empty())
        PS_CUDA(cudaMemcpyAsync(dRemap_.get(), hRemap_.data(), hRemap_.size() * sizeof(RemapItem),
                                cudaMemcpyHostToDevice, st));
    PS_CUDA(cudaMemcpyAsync(dLinear_.get(), lin.data(), lin.size() * sizeof(LinearItem), cudaMemcpyHostToDevice, st));
    const size_t tiles = std::max<size_t>(1, hRemap_.size());
    maps_.alloc(tiles * kRemapTW * kRemapTH * sizeof(float2));
    linW_.alloc(tiles * kRemapTW * kRemapTH * sizeof(float));
    if (!hRemap_.empty())
        PS_CUDA(launchCompactMaps(xmap, ymap, W, H, (long long)npx, dRemap_.as<RemapItem>(), (int)hRemap_.size(),
                                  maps_.as<float2>(), st));
    // weights (getWeightsLinearBlend32F)
    const std::vector<int> taps = gaussTaps(radius);
    DevBuf dTaps(taps.size() * sizeof(int));
    PS_CUDA(cudaMemcpyAsync(dTaps.get(), taps.data(), dTaps.bytes(), cudaMemcpyHostToDevice, st));
    {
        DevBuf rows(n * npx * 4), dist(n * npx), wFull(n * npx * 4);
        PS_CUDA(launchLinearWeights(seam, cov, n, W, H, dTaps.as<int>(), radius, rows.as<int32_t>(), dist.as<uint8_t>(),
                                    wFull.as<float>(), dRemap_.as<RemapItem>(), (int)hRemap_.size(), linW_.as<float>(),
                                    st));
        PS_CUDA(cudaStreamSynchronize(st));
    }
    RigDev d;
    std::memset(&d, 0, sizeof d);
    d.n = n;
    d.W = W;
    d.H = H;
    d.full = full_;
    d.srcW = srcW_;
    d.srcH = srcH_;
    d.maps = maps_.as<float2>();
    d.remapItems = dRemap_.as<RemapItem>();
    d.numRemapItems = (int)hRemap_.size();
    d.linWeights = linW_.as<float>();
    d.tailDown = d.tailBlend = 1;
    d.lv[0].w = W;
    d.lv[0].h = H;
    d.lv[0].pitch = geom_[0].pitch;
    RigDev ds[kIoSlots];
    for (int k = 0; k < slots_; k++) ds[k] = d;
    dDesc_.alloc(sizeof(RigDev) * slots_);
    PS_CUDA(cudaMemcpyAsync(dDesc_.get(), ds, sizeof(RigDev) * slots_, cudaMemcpyHostToDevice, st));
    PS_CUDA(cudaStreamSynchronize(st));
    tailDown_ = tailBlend_ = 1;  // no pyramid
    gen_ = g_generation++;
}

void Rig::imagesToLevel0(const void* const* images, const long long* pitches, int fmt, int slot, cudaStream_t st)
{
    toLevel0(images, pitches, fmt, 0, n_, slot, st);
}

void Rig::imageToLevel0(const void* image, long long pitch, int fmt, int cam, int slot, cudaStream_t st)
{
    if (cam < 0 || cam >= n_) fail(PS_EINVAL, "camera %d out of range 0..%d", cam, n_ - 1);
    toLevel0(&image, &pitch, fmt, cam, 1, slot, st);
}

void Rig::zeroLevel0(int cam, int slot, cudaStream_t st)
{
    const LevelGeom& g = geom_[0];
    PS_CUDA(cudaMemsetAsync(lv_[0].G[slot].as<uchar4>() + (size_t)cam * g.pitch * g.h, 0,
                            (size_t)g.pitch * g.h * sizeof(uchar4), st));
}

void Rig::toLevel0(const void* const* images, const long long* pitches, int fmt, int cam0, int count, int slot,
                   cudaStream_t st)
{
    const size_t n = count;
    std::vector<uint8_t> args((sizeof(void*) + sizeof(long long)) * n);
    std::memcpy(args.data(), images, sizeof(void*) * n);
    std::memcpy(args.data() + sizeof(void*) * n, pitches, sizeof(long long) * n);
    PS_CUDA(cudaMemcpyAsync(imgArgs_.get(), args.data(), args.size(), cudaMemcpyHostToDevice, st));
    PS_CUDA(cudaMemsetAsync(status_.get(), 0, sizeof(int), st));
    const LevelGeom& g = geom_[0];
    const size_t npx = (size_t)W_ * H_;
    PS_CUDA(launchImagesToLevel0(imgArgs_.as<const void* const>(),
                                 reinterpret_cast<const long long*>(imgArgs_.as<uint8_t>() + sizeof(void*) * n), fmt,
                                 count, W_, H_, covDev_.as<uint8_t>() + cam0 * npx, (long long)npx,
                                 lv_[0].G[slot].as<uchar4>() + (size_t)cam0 * g.pitch * g.h, g.pitch,
                                 (long long)g.pitch * g.h, status_.as<int>(), st));
    int status = 0;
    PS_CUDA(cudaMemcpyAsync(&status, status_.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaStreamSynchronize(st));
    if (status & 1) fail(PS_EINVAL, "an int16 input value lies outside 0..255");
    if (status & 2) fail(PS_EINVAL, "an input image is non-zero where its coverage mask is zero");
}

void Rig::exportState(int what, int cam, int level, void* host, long long bytes) const
{
    if (!ready()) fail(PS_ESTATE, "not prepared");
    if (cam < 0 || cam >= n_) fail(PS_EINVAL, "camera %d out of range", cam);
    const size_t npx = (size_t)W_ * H_;
    if (what == 7) {  // level 0 of the last run (the remap's output; uint8 x4, the fourth byte 0)
        if ((size_t)bytes < npx * 4) fail(PS_EINVAL, "buffer too small");
        const_cast<Rig*>(this)->waitIdle();  // the runs are on the render's own streams
        const LevelGeom& g = geom_[0];
        PS_CUDA(cudaMemcpy2D(host, (size_t)W_ * 4, lv_[0].G[lastSlot_].as<uchar4>() + (size_t)cam * g.pitch * g.h,
                             (size_t)g.pitch * 4, (size_t)W_ * 4, H_, cudaMemcpyDeviceToHost));
        return;
    }
    if (what == 0 || what == 1) {
        if (!hasMaps_) fail(PS_EINVAL, "no maps (prepared from masks)");
        if (mapFree_) fail(PS_EINVAL, "map-free render: the maps are not resident");
        if ((size_t)bytes < npx * 4) fail(PS_EINVAL, "buffer too small");
        float* out = static_cast<float*>(host);
        std::fill(out, out + npx, -1.f);
        std::vector<float2> m(hRemap_.size() * kRemapTW * kRemapTH);
        if (!m.empty()) PS_CUDA(cudaMemcpy(m.data(), maps_.get(), m.size() * sizeof(float2), cudaMemcpyDeviceToHost));
        for (const RemapItem& it : hRemap_) {
            if (it.cam != cam) continue;
            for (int k = 0; k < kRemapTW * kRemapTH; k++) {
                const int x = it.tx * kRemapTW + (k % kRemapTW), y = it.ty * kRemapTH + (k / kRemapTW);
                if (x < W_ && y < H_) {
                    const float2 v = m[(size_t)it.mapTile * kRemapTW * kRemapTH + k];
                    out[(size_t)y * W_ + x] = what == 0 ? v.x : v.y;
                }
            }
        }
        return;
    }
    if (what == 2 || what == 3) {
        if ((size_t)bytes < npx) fail(PS_EINVAL, "buffer too small");
        const std::vector<uint8_t>& bits = what == 2 ? covBits_ : seamBits_;
        uint8_t* out = static_cast<uint8_t*>(host);
        const size_t base = (size_t)cam * npx;
        for (size_t i = 0; i < npx; i++) out[i] = (bits[(base + i) >> 3] >> ((base + i) & 7)) & 1 ? 255 : 0;
        return;
    }
    if (what == 6) {  // linear-blend weights (float per pixel, 0 outside the camera's tiles)
        if (!linear_) fail(PS_EINVAL, "no linear-blend weights (multiband mode)");
        if ((size_t)bytes < npx * 4) fail(PS_EINVAL, "buffer too small");
        float* out = static_cast<float*>(host);
        std::fill(out, out + npx, 0.f);
        std::vector<float> w(hRemap_.size() * kRemapTW * kRemapTH);
        if (!w.empty()) PS_CUDA(cudaMemcpy(w.data(), linW_.get(), w.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (const RemapItem& it : hRemap_) {
            if (it.cam != cam) continue;
            for (int k = 0; k < kRemapTW * kRemapTH; k++) {
                const int x = it.tx * kRemapTW + (k % kRemapTW), y = it.ty * kRemapTH + (k / kRemapTW);
                if (x < W_ && y < H_) out[(size_t)y * W_ + x] = w[(size_t)it.mapTile * kRemapTW * kRemapTH + k];
            }
        }
        return;
    }
    if (what == 4 || what == 5) {
        if (linear_) fail(PS_EINVAL, "no pyramids (linear-blend mode)");
        if (level < 0 || level > L_ || (what == 5 && level == 0)) fail(PS_EINVAL, "level %d out of range", level);
        const LevelGeom& g = geom_[level];
        const size_t cnt = (size_t)g.w * g.h;
        const size_t esz = what == 4 ? 2 : 4;
        if ((size_t)bytes < cnt * esz) fail(PS_EINVAL, "buffer too small");
        std::vector<uint16_t> tmp(cnt);
        const DevBuf& src = what == 4 ? lv_[level].Wt : lv_[level].Am;
        PS_CUDA(cudaMemcpy2D(tmp.data(), g.w * 2, src.as<uint16_t>() + (size_t)cam * g.pitch * g.h, g.pitch * 2,
                             g.w * 2, g.h, cudaMemcpyDeviceToHost));
        if (what == 4) std::memcpy(host, tmp.data(), cnt * 2);
        else {
            int32_t* out = static_cast<int32_t*>(host);
            for (size_t i = 0; i < cnt; i++) out[i] = (int32_t)tmp[i] * 256;
        }
        return;
    }
    fail(PS_EINVAL, "unknown export %d", what);
}

void Rig::exportCollapsed(int level, int16_t* host, long long bytes, cudaStream_t st) const
{
    if (!ready()) fail(PS_ESTATE, "not prepared");
    if (level < 1 || level > L_) fail(PS_EINVAL, "level %d out of range 1..%d", level, L_);
    const LevelGeom& g = geom_[level];
    if ((size_t)bytes < (size_t)g.w * g.h * 8) fail(PS_EINVAL, "buffer too small");
    PS_CUDA(cudaMemcpy2DAsync(host, (size_t)g.w * 8, lv_[level].C[lastSlot_].get(), (size_t)g.pitch * 8, (size_t)g.w * 8, g.h,
                              cudaMemcpyDeviceToHost, st));
    PS_CUDA(cudaStreamSynchronize(st));
}

double Rig::stepBytes(int kind, int level) const
{
    double b = 0;
    if (kind == 4) {
        // map (8 B) and weight (4 B) per covered tile pixel, every covering frame once, the canvas out
        std::vector<char> used(n_, 0);
        for (const RemapItem& it : hRemap_) {
            const int tw = std::min(kRemapTW, W_ - it.tx * kRemapTW), th = std::min(kRemapTH, H_ - it.ty * kRemapTH);
            b += (double)tw * th * 12;
            used[it.cam] = 1;
        }
        for (int c = 0; c < n_; c++)
            if (used[c]) b += (double)srcW_ * srcH_ * 4;
        return b + (double)W_ * H_ * 4;
    }
    if (kind == 3) {
        for (int J = tailDown_; J <= L_; J++) b += stepBytes(1, J);
        for (int j = tailBlend_; j <= L_; j++) b += stepBytes(2, j);
        return b;
    }
    if (kind == 0) {
        // map (8 B) in, G0 (4 B) out per tile pixel, every covering camera's frame in once
        std::vector<char> used(n_, 0);
        for (const RemapItem& it : hRemap_) {
            const int tw = std::min(kRemapTW, W_ - it.tx * kRemapTW), th = std::min(kRemapTH, H_ - it.ty * kRemapTH);
            b += (double)tw * th * 12;
            used[it.cam] = 1;
        }
        for (int c = 0; c < n_; c++)
            if (used[c]) b += (double)srcW_ * srcH_ * 4;
        return b;
    }
    if (kind == 1) {
        // per output pixel: 4 input pixels (uchar4), the alpha divisor (2 B), the output (4 B)
        const LevelGeom& g = geom_[level];
        for (int k = downOff_[level]; k < downOff_[level] + downCnt_[level]; k++) {
            const DownItem& it = hDown_[k];
            const int tw = std::min(kDownTW, g.w - it.tx * kDownTW), th = std::min(kDownTH, g.h - it.ty * kDownTH);
            b += (double)tw * th * (16 + 2 + 4);
        }
        return b;
    }
    // blend: per camera in the tile's list weight (2 B) + G_j (4 B) + a quarter of G_{j+1} (1 B);
    // a quarter of C_{j+1} (2 B); out C_j (8 B) or the canvas (4 B)
    const LevelGeom& g = geom_[level];
    for (int k = blendOff_[level]; k < blendOff_[level] + blendCnt_[level]; k++) {
        const BlendItem& it = hBlend_[k];
        const int tw = std::min(kBlendTW, g.w - it.tx * kBlendTW), th = std::min(kBlendTH, g.h - it.ty * kBlendTH);
        if (level == 0 && it.cls == 0) { b += (double)tw * th * 4; continue; }
        const double perCam = level < L_ ? 7 : 6;
        b += (double)tw * th * (it.camCnt * perCam + (level < L_ ? 2 : 0) + (level > 0 ? 8 : 4) +
                                (level == 0 && it.cls == 2 ? 1 : 0));
    }
    return b;
}

double Rig::algorithmicBytes(int bin, int bout) const
{
    if (linear_)  // frames in, map (8 B) and weight (4 B) per covered pixel, canvas out
        return (double)n_ * srcW_ * srcH_ * bin + (double)covCount_ * 12 + (double)W_ * H_ * bout;
    return (double)n_ * srcW_ * srcH_ * bin + (double)covCount_ * 8 + (double)weightCount_ * 2 +
           (double)alphaCount_ * 4 + (double)W_ * H_ * bout;
}

// ---- Profiler -------------------------------------------------------------------------
Profiler::~Profiler()
{
    for (auto& r : recs_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : free_) cudaEventDestroy(e);
}

void Profiler::enable(bool on)
{
    if (on && !on_) {
        collect();
        agg_.clear();
    }
    on_ = on;
}

cudaEvent_t Profiler::event()
{
    if (!free_.empty()) {
        cudaEvent_t e = free_.back();
        free_.pop_back();
        return e;
    }
    cudaEvent_t e;
    PS_CUDA(cudaEventCreate(&e));
    return e;
}

void Profiler::record(int kind, int level, double bytes, cudaEvent_t a, cudaEvent_t b)
{
    recs_.push_back({kind, level, bytes, a, b});
}

void Profiler::collect()
{
    for (auto& r : recs_) {
        PS_CUDA(cudaEventSynchronize(r.b));
        float ms = 0;
        PS_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        auto key = std::make_pair(r.kind, r.level);
        auto it = std::find_if(agg_.begin(), agg_.end(), [&](const auto& p) { return p.first == key; });
        if (it == agg_.end()) { agg_.push_back({key, Agg()}); it = agg_.end() - 1; }
        it->second.launches++;
        it->second.ms += ms;
        it->second.bytes += r.bytes;
        free_.push_back(r.a);
        free_.push_back(r.b);
    }
    recs_.clear();
}

void Profiler::read(int kind, int level, long long* launches, double* ms, double* bytes)
{
    collect();
    long long l = 0;
    double t = 0, b = 0;
    for (const auto& p : agg_)
        if (p.first.first == kind && (level < 0 || p.first.second == level)) {
            l += p.second.launches;
            t += p.second.ms;
            b += p.second.bytes;
        }
    if (launches) *launches = l;
    if (ms) *ms = t;
    if (bytes) *bytes = b;
}

// ---- Plan ---------------------------------------------------------------------------
void Plan::dropGraph()
{
    for (IoSlot& sl : io_) {
        if (sl.graph) cudaGraphExecDestroy(sl.graph);
        sl.graph = nullptr;
    }
}

void Plan::ensureStreams()
{
    if (sIn_) return;
    PS_CUDA(cudaStreamCreateWithFlags(&sIn_, cudaStreamNonBlocking));
    for (cudaStream_t& c : sComp_) PS_CUDA(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
    PS_CUDA(cudaStreamCreateWithFlags(&sOut_, cudaStreamNonBlocking));
    PS_CUDA(cudaStreamCreateWithFlags(&capStream_, cudaStreamNonBlocking));
    PS_CUDA(cudaEventCreateWithFlags(&callerEv_, cudaEventDisableTiming));
    for (IoSlot& sl : io_) {
        PS_CUDA(cudaEventCreateWithFlags(&sl.argsCopied, cudaEventDisableTiming));
        PS_CUDA(cudaEventCreateWithFlags(&sl.computed, cudaEventDisableTiming));
        PS_CUDA(cudaEventCreateWithFlags(&sl.downloaded, cudaEventDisableTiming));
    }
}

// Wait until no run of this plan is in flight (before its buffers change).
void Plan::quiesce()
{
    for (cudaStream_t st : {sIn_, sOut_})
        if (st) PS_CUDA(cudaStreamSynchronize(st));
    for (cudaStream_t st : sComp_)
        if (st) PS_CUDA(cudaStreamSynchronize(st));
}

void Plan::bind(const std::vector<Rig*>& rigs)
{
    const int nr = (int)rigs.size();
    int maxL = 0;
    for (Rig* r : rigs) {
        if (!r || !r->ready()) fail(PS_ESTATE, "render not prepared");
        maxL = std::max(maxL, r->numLevels());
    }
    quiesce();
    dropGraph();
    rigs_ = rigs;
    gens_.clear();
    for (Rig* r : rigs) gens_.push_back(r->generation());
    lutOff_.clear();
    size_t off = (sizeof(FrameDev) * nr + 15) / 16 * 16;  // LUTs 16-byte aligned for bulk copies
    for (Rig* r : rigs) {
        lutOff_.push_back(off);
        off += (size_t)r->numImages() * 768;
    }
    segOff_ = (off + 15) / 16 * 16;

    steps_.clear();
    segs_.clear();
    segRig_.clear();
    maxCams_ = 0;
    for (Rig* r : rigs) maxCams_ = std::max(maxCams_, r->numImages());
    // launch widths shared by the rigs of a launch: the widest any rig asks
    // for, 0 (as many as fit) counting as widest
    auto widest = [&](auto field) {
        int v = -1;
        for (Rig* r : rigs) {
            const int x = field(r->shape());
            if (x == 0) return 0;
            v = std::max(v, x);
        }
        return v < 0 ? 0 : v;
    };
    tailCluster_ = widest([](const LaunchShape& s) { return s.tailCluster; });
    for (int k = 0; k < 3; k++) perSm_[k] = widest([k](const LaunchShape& s) { return s.ctasPerSm[k]; });
    remapDefer_ = false;  // deferred when any rig of the launch asks for it
    for (Rig* r : rigs) remapDefer_ = remapDefer_ || r->shape().remapDefer;
    probe_ = 0;
    for (Rig* r : rigs) probe_ = std::max(probe_, r->waitProbe());
    auto addStep = [&](int kind, const std::vector<std::pair<int, std::pair<const void*, int>>>& parts, int step) {
        Step s{kind, (int)segs_.size(), 0, 0, -1, 0.0};
        for (const auto& p : parts) {
            if (p.second.second <= 0) continue;
            // frame pointer holds the FrameDev offset until the buffer is known
            segRig_.push_back(p.first);
            segs_.push_back({p.second.first, rigs[p.first]->deviceDesc(),
                             reinterpret_cast<const FrameDev*>(sizeof(FrameDev) * p.first), p.second.second, s.total});
            s.total += p.second.second;
            const Rig* rg = rigs[p.first];
            const int lvl = kind == 0 || kind == 4 ? 0 : (kind == 1 ? step : rg->tailBlend() - 1 - step);
            if (s.level < 0) s.level = lvl;
            s.bytes += rg->stepBytes(kind == 6 ? 2 : kind, lvl);
        }
        s.nsegs = (int)segs_.size() - s.segOff;
        if (s.total > 0) steps_.push_back(s);
    };
    std::vector<std::pair<int, std::pair<const void*, int>>> parts;
    for (int r = 0; r < nr; r++)
        if (rigs[r]->linear()) parts.push_back({r, {rigs[r]->linearItems(), rigs[r]->numLinearItems()}});
    addStep(4, parts, 0);
    parts.clear();
    for (int r = 0; r < nr; r++)
        if (!rigs[r]->linear()) parts.push_back({r, {rigs[r]->remapItems(), rigs[r]->numRemapItems()}});
    addStep(0, parts, 0);
    int remapTotal = 0;
    if (remapDefer_ && !steps_.empty() && steps_.back().kind == 0) {  // its exact recompute, same segments
        Step f = steps_.back();
        f.kind = 7;
        f.bytes = 0;
        remapTotal = f.total;
        steps_.push_back(f);
    }
    for (int J = 1; J <= maxL; J++) {
        parts.clear();
        for (int r = 0; r < nr; r++)
            if (J < rigs[r]->tailDown()) parts.push_back({r, {rigs[r]->downItems(J), rigs[r]->numDownItems(J)}});
        addStep(1, parts, J);
    }
    {
        // the tail: one cluster per rig that has one (segment count 1)
        Step s{3, (int)segs_.size(), 0, 0, -1, 0.0};
        for (int r = 0; r < nr; r++) {
            if (rigs[r]->linear() || !rigs[r]->hasTail()) continue;
            segRig_.push_back(r);
            segs_.push_back({nullptr, rigs[r]->deviceDesc(), reinterpret_cast<const FrameDev*>(sizeof(FrameDev) * r), 1,
                             s.total});
            s.total += 1;
            if (s.level < 0) s.level = rigs[r]->tailBlend();
            s.bytes += rigs[r]->stepBytes(3, 0);
        }
        s.nsegs = (int)segs_.size() - s.segOff;
        if (s.total > 0) steps_.push_back(s);
    }
    int maxB = 0;
    for (Rig* r : rigs)
        if (!r->linear()) maxB = std::max(maxB, r->tailBlend());
    for (int s = 0; s < maxB; s++) {
        // levels above 0 with few tiles go to k_blend_small (two halves per tile)
        std::vector<std::pair<int, std::pair<const void*, int>>> small;
        parts.clear();
        for (int r = 0; r < nr; r++) {
            if (rigs[r]->linear()) continue;
            const int j = rigs[r]->tailBlend() - 1 - s;
            if (j < 0) continue;
            const int cnt = rigs[r]->numBlendItems(j);
            if (j > 0 && cnt <= rigs[r]->shape().smallBlendMaxItems) small.push_back({r, {rigs[r]->blendItems(j), 2 * cnt}});
            else parts.push_back({r, {rigs[r]->blendItems(j), cnt}});
        }
        const size_t before = steps_.size();
        addStep(6, small, s);
        addStep(2, parts, s);
        for (size_t k = before; k < steps_.size(); k++) steps_[k].early = s > 0;
    }
    // one work counter per step after the segments, zeroed in every run's staged copy
    // and the remap's tie count after them
    counterOff_ = (segOff_ + segs_.size() * sizeof(Segment) + 15) / 16 * 16;
    const size_t need = counterOff_ + (steps_.size() + 1) * sizeof(int);
    for (IoSlot& sl : io_)
        if (need > sl.dArgs.bytes()) {
            const size_t cap = need + need / 2;
            sl.dArgs.alloc(cap);
            sl.stage.alloc(cap);
        }
    stageBytes_ = counterOff_ + (steps_.size() + 1) * sizeof(int);
    for (IoSlot& sl : io_)
        if ((size_t)remapTotal * kRemapTiesPerTile * sizeof(RemapTie) > sl.ties.bytes())
            sl.ties.alloc((size_t)remapTotal * kRemapTiesPerTile * sizeof(RemapTie));
}

Plan::~Plan()
{
    for (cudaStream_t st : {sIn_, sOut_})
        if (st) cudaStreamSynchronize(st);
    for (cudaStream_t st : sComp_)
        if (st) cudaStreamSynchronize(st);
    dropGraph();
    for (cudaStream_t st : {sIn_, sOut_, capStream_})
        if (st) cudaStreamDestroy(st);
    for (cudaStream_t st : sComp_)
        if (st) cudaStreamDestroy(st);
    if (callerEv_) cudaEventDestroy(callerEv_);
    for (IoSlot& sl : io_)
        for (cudaEvent_t e : {sl.argsCopied, sl.computed, sl.downloaded})
            if (e) cudaEventDestroy(e);
}

bool Plan::matches(const std::vector<Rig*>& rigs) const
{
    if (rigs.size() != rigs_.size()) return false;
    for (size_t i = 0; i < rigs.size(); i++)
        if (rigs[i] != rigs_[i] || rigs[i]->generation() != gens_[i]) return false;
    return true;
}

void Plan::launchAll(const IoSlot& slot, cudaStream_t st, int srcFmt, Profiler* prof)
{
    const Segment* segs = reinterpret_cast<const Segment*>(static_cast<const uint8_t*>(slot.dArgs.get()) + segOff_);
    int* counters = reinterpret_cast<int*>(static_cast<uint8_t*>(slot.dArgs.get()) + counterOff_);
    for (size_t si = 0; si < steps_.size(); si++) {
        const Step& s = steps_[si];
        const Segment* p = segs + s.segOff;
        static const char* const kRangeName[] = {"ps.remap", "ps.pyrdown", "ps.blend", "ps.tail",
                                                 "ps.linear", "ps.cvt", "ps.blend_small", "ps.remap_fix"};
        NvtxRange range(kRangeName[s.kind >= 0 && s.kind <= 7 ? s.kind : 5]);
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof) {
            a = prof->event();
            b = prof->event();
            PS_CUDA(cudaEventRecord(a, st));
        }
        int* tieCount = counters + steps_.size();  // the remap's count of listed near-tie pixels
        if (s.kind == 0)
            PS_CUDA(launchRemap(p, s.nsegs, s.total, perSm_[0], counters + si, tieCount, slot.ties.as<RemapTie>(),
                                remapDefer_, srcFmt, st));
        else if (s.kind == 7) PS_CUDA(launchRemapFix(p, s.nsegs, s.total, tieCount, slot.ties.as<RemapTie>(), st));
        else if (s.kind == 1) PS_CUDA(launchPyrDown(p, s.nsegs, s.total, perSm_[1], st));
        else if (s.kind == 2) PS_CUDA(launchBlend(p, s.nsegs, s.total, perSm_[2], counters + si, probe_, s.early, st));
        else if (s.kind == 3) PS_CUDA(launchTail(p, s.nsegs, tailCluster_, st));
        else if (s.kind == 6) PS_CUDA(launchBlendSmall(p, s.nsegs, s.total, s.early, st));
        else PS_CUDA(launchLinear(p, s.nsegs, s.total, maxCams_, st));
        if (prof) {
            PS_CUDA(cudaEventRecord(b, st));
            prof->record(s.kind, s.level, s.bytes, a, b);
        }
    }
}

static int bytesPerPixel(int fmt) { return fmt == PS_FMT_BGR24 ? 3 : 4; }

// One run: copy-in (host frames, the staged arguments), compute (one stream
// per slot), copy-out (host canvases).  Runs take the kIoSlots slots of
// arguments and rig state in turn and wait only for the previous run on the
// same slot, so with host buffers on both sides consecutive runs overlap.
// With any device input or output the run also waits for the caller's
// stream.  The caller's stream waits for the run's completion.
void Plan::run(const std::vector<FrameInput>& in, cudaStream_t st, bool useGraph, Profiler* prof)
{
    NvtxRange range("ps.run");
    if (prof && !prof->on()) prof = nullptr;
    if (prof) useGraph = false;
    if (in.size() != rigs_.size()) fail(PS_EINVAL, "plan input count mismatch");
    ensureStreams();
    const int si = nextIo_;
    IoSlot& S = io_[si];
    bool hostOnly = true;
    for (const FrameInput& f : in) {
        Rig* rig = rigs_[&f - in.data()];
        if (f.psrc) {
            rig->ensurePlanar();  // before any work of this run is queued
            for (int i = 0; i < rig->numImages(); i++)
                if (f.psrc[i].location != PS_MEM_HOST) hostOnly = false;
        } else if (!f.src) {
            hostOnly = false;  // level 0 written on the caller's stream
        } else {
            for (int i = 0; i < rig->numImages(); i++)
                if (f.src[i].location != PS_MEM_HOST) hostOnly = false;
        }
        if ((f.ydst ? f.ydst->location : f.dst->location) != PS_MEM_HOST) hostOnly = false;
    }
    if (S.used) PS_CUDA(cudaEventSynchronize(S.argsCopied));  // the slot's pinned stage is free again
    PS_CUDA(cudaEventRecord(callerEv_, st));
    // each rig's state slot (pyramids, I/O staging); without sources it is
    // the slot imagesToLevel0 just filled (peekSlot)
    std::vector<int> rs(rigs_.size());
    for (size_t r = 0; r < rigs_.size(); r++) rs[r] = rigs_[r]->acquireSlot();
    cudaStream_t comp = sComp_[si];

    // ---- copy-in: after the previous kernels on the rigs' slots (inputs, pyramids) and on this args slot
    if (!hostOnly) PS_CUDA(cudaStreamWaitEvent(sIn_, callerEv_, 0));
    if (S.used) PS_CUDA(cudaStreamWaitEvent(sIn_, S.computed, 0));
    for (size_t r = 0; r < rigs_.size(); r++) PS_CUDA(cudaStreamWaitEvent(sIn_, rigs_[r]->slotComputed(rs[r]), 0));
    uint8_t* stage = S.stage.as<uint8_t>();
    uint8_t* dArgs = S.dArgs.as<uint8_t>();
    std::vector<YuvFrames> cvt;  // decoder frames converted into the slots' BGR32 staging
    double cvtBytes = 0;
    int srcFmt = -1;  // the format all rigs' sources share, else 0
    for (size_t r = 0; r < rigs_.size(); r++) {
        Rig* rig = rigs_[r];
        const FrameInput& f = in[r];
        FrameDev fd;
        std::memset(&fd, 0, sizeof fd);
        const int n = rig->numImages();
        if (f.psrc) {
            YuvFrames y;
            std::memset(&y, 0, sizeof y);
            y.w = rig->srcW();
            y.h = rig->srcH();
            const size_t w = y.w, h = y.h;
            fd.srcFmt = PS_FMT_BGR32;
            for (int i = 0; i < n; i++) {
                const ps_planar_image& s = f.psrc[i];
                // a host frame given for several cameras goes up and is converted once
                int same = -1;
                for (int q = 0; q < i && same < 0 && s.location == PS_MEM_HOST; q++)
                    if (f.psrc[q].location == PS_MEM_HOST && f.psrc[q].format == s.format &&
                        f.psrc[q].planes[0] == s.planes[0] && f.psrc[q].planes[1] == s.planes[1] &&
                        f.psrc[q].planes[2] == s.planes[2] && f.psrc[q].pitches[0] == s.pitches[0] &&
                        f.psrc[q].pitches[1] == s.pitches[1] && f.psrc[q].pitches[2] == s.pitches[2])
                        same = q;
                if (same >= 0) {
                    fd.src[i] = fd.src[same];
                    fd.srcPitch[i] = fd.srcPitch[same];
                    continue;
                }
                YuvFrame& F = y.frame[y.n++];
                F.fmt = s.format;
                const bool nv12 = s.format == PS_FMT_NV12;
                if (s.location == PS_MEM_HOST) {  // packed planes in the slot's staging
                    uint8_t* base = rig->planarBuffer(i, rs[r]);
                    PS_CUDA(cudaMemcpy2DAsync(base, w, s.planes[0], s.pitches[0], w, h, cudaMemcpyHostToDevice, sIn_));
                    F.y = base;
                    F.yPitch = (long long)w;
                    F.u = base + w * h;
                    if (nv12) {
                        F.uPitch = (long long)w;
                        PS_CUDA(cudaMemcpy2DAsync(base + w * h, w, s.planes[1], s.pitches[1], w, h / 2,
                                                  cudaMemcpyHostToDevice, sIn_));
                    } else {
                        F.uPitch = F.vPitch = (long long)(w / 2);
                        F.v = F.u + w * h / 4;
                        PS_CUDA(cudaMemcpy2DAsync(base + w * h, w / 2, s.planes[1], s.pitches[1], w / 2, h / 2,
                                                  cudaMemcpyHostToDevice, sIn_));
                        PS_CUDA(cudaMemcpy2DAsync(base + w * h + w * h / 4, w / 2, s.planes[2], s.pitches[2], w / 2,
                                                  h / 2, cudaMemcpyHostToDevice, sIn_));
                    }
                } else {
                    F.y = static_cast<const uint8_t*>(s.planes[0]);
                    F.yPitch = s.pitches[0];
                    F.u = static_cast<const uint8_t*>(s.planes[1]);
                    F.uPitch = s.pitches[1];
                    if (!nv12) {
                        F.v = static_cast<const uint8_t*>(s.planes[2]);
                        F.vPitch = s.pitches[2];
                    }
                }
                F.dst = rig->inputBuffer(i, rs[r]);
                F.dstPitch = rig->inputPitch();
                fd.src[i] = F.dst;
                fd.srcPitch[i] = rig->inputPitch();
            }
            cvt.push_back(y);
            cvtBytes += (double)y.n * w * h * (1.5 + 4);
        } else if (f.src) {
            fd.srcFmt = f.src[0].format;
            for (int i = 0; i < n; i++) {
                const ps_image& s = f.src[i];
                if (s.location == PS_MEM_HOST) {
                    // a host frame given for several cameras (both lenses of a
                    // dual-fisheye frame) goes up once
                    int same = -1;
                    for (int q = 0; q < i && same < 0; q++)
                        if (f.src[q].location == PS_MEM_HOST && f.src[q].data == s.data && f.src[q].pitch == s.pitch)
                            same = q;
                    if (same >= 0) {
                        fd.src[i] = fd.src[same];
                        fd.srcPitch[i] = fd.srcPitch[same];
                        continue;
                    }
                    const size_t rowBytes = (size_t)s.width * bytesPerPixel(s.format);
                    PS_CUDA(cudaMemcpy2DAsync(rig->inputBuffer(i, rs[r]), rig->inputPitch(), s.data, s.pitch, rowBytes,
                                              s.height, cudaMemcpyHostToDevice, sIn_));
                    fd.src[i] = rig->inputBuffer(i, rs[r]);
                    fd.srcPitch[i] = rig->inputPitch();
                } else {
                    fd.src[i] = static_cast<const uint8_t*>(s.data);
                    fd.srcPitch[i] = s.pitch;
                }
            }
        }
        uint8_t* lut = stage + lutOff_[r];
        if (f.luts) std::memcpy(lut, f.luts, (size_t)n * 768);
        else
            for (int i = 0; i < n * 3; i++)
                for (int v = 0; v < 256; v++) lut[i * 256 + v] = (uint8_t)v;
        fd.luts = dArgs + lutOff_[r];
        if (f.ydst) {
            const ps_planar_image& d = *f.ydst;
            if (d.location == PS_MEM_HOST) {  // planes staged tightly in the output buffer, then downloaded
                const size_t luma = (size_t)d.width * d.height;
                fd.out = rig->outputBuffer(rs[r]);
                fd.outPitch = d.width;
                fd.outU = fd.out + luma;
                fd.outCPitch = d.format == PS_FMT_NV12 ? d.width : d.width / 2;
                fd.outV = fd.outU + luma / 4;
                fd.outVPitch = d.width / 2;
            } else {
                fd.out = static_cast<uint8_t*>(d.planes[0]);
                fd.outPitch = d.pitches[0];
                fd.outU = static_cast<uint8_t*>(d.planes[1]);
                fd.outCPitch = d.pitches[1];
                fd.outV = static_cast<uint8_t*>(d.planes[2]);
                fd.outVPitch = d.pitches[2];
            }
            fd.outFmt = d.format;
        } else {
            const ps_image& d = *f.dst;
            if (d.location == PS_MEM_HOST) {
                fd.out = rig->outputBuffer(rs[r]);
                fd.outPitch = (long long)d.width * bytesPerPixel(d.format);
            } else {
                fd.out = static_cast<uint8_t*>(d.data);
                fd.outPitch = d.pitch;
            }
            fd.outFmt = d.format;
        }
        fd.status = rig->statusWord();
        srcFmt = srcFmt < 0 || srcFmt == fd.srcFmt ? fd.srcFmt : 0;
        std::memcpy(stage + sizeof(FrameDev) * r, &fd, sizeof fd);
    }
    if (!segs_.empty()) {
        Segment* sg = reinterpret_cast<Segment*>(stage + segOff_);
        const uintptr_t base = reinterpret_cast<uintptr_t>(dArgs);
        for (size_t k = 0; k < segs_.size(); k++) {
            sg[k] = segs_[k];
            sg[k].frame = reinterpret_cast<const FrameDev*>(base + reinterpret_cast<uintptr_t>(segs_[k].frame));
            sg[k].rig = rigs_[segRig_[k]]->deviceDesc(rs[segRig_[k]]);
        }
    }
    std::memset(stage + counterOff_, 0, (steps_.size() + 1) * sizeof(int));
    PS_CUDA(cudaMemcpyAsync(dArgs, stage, stageBytes_, cudaMemcpyHostToDevice, sIn_));
    PS_CUDA(cudaEventRecord(S.argsCopied, sIn_));

    // ---- compute: one stream per args slot, so two runs' kernels can overlap
    PS_CUDA(cudaStreamWaitEvent(comp, S.argsCopied, 0));
    if (!hostOnly) PS_CUDA(cudaStreamWaitEvent(comp, callerEv_, 0));
    for (size_t r = 0; r < rigs_.size(); r++)  // the output staging has been read out
        PS_CUDA(cudaStreamWaitEvent(comp, rigs_[r]->slotDownloaded(rs[r]), 0));
    for (const YuvFrames& y : cvt) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof) {
            a = prof->event();
            b = prof->event();
            PS_CUDA(cudaEventRecord(a, comp));
        }
        PS_CUDA(launchYuvToBgr32(y, comp));
        if (prof) {
            PS_CUDA(cudaEventRecord(b, comp));
            prof->record(5, 0, cvtBytes / cvt.size(), a, b);
        }
    }
    srcFmt = srcFmt == PS_FMT_BGR32 ? PS_FMT_BGR32 : 0;  // the formats the remap is specialised for
    if (useGraph) {
        if (S.graph && S.graphFmt != srcFmt) {  // re-record for the other format, after the slot's last run
            if (S.used) PS_CUDA(cudaEventSynchronize(S.computed));
            PS_CUDA(cudaGraphExecDestroy(S.graph));
            S.graph = nullptr;
        }
        if (!S.graph) {
            S.graphFmt = srcFmt;
            cudaGraph_t g = nullptr;
            PS_CUDA(cudaStreamBeginCapture(capStream_, cudaStreamCaptureModeThreadLocal));
            try {
                launchAll(S, capStream_, srcFmt);
            } catch (...) {
                cudaStreamEndCapture(capStream_, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            PS_CUDA(cudaStreamEndCapture(capStream_, &g));
            const cudaError_t e = cudaGraphInstantiate(&S.graph, g, 0);
            cudaGraphDestroy(g);
            PS_CUDA(e);
        }
        PS_CUDA(cudaGraphLaunch(S.graph, comp));
    } else {
        launchAll(S, comp, srcFmt, prof);
    }
    PS_CUDA(cudaEventRecord(S.computed, comp));
    for (size_t r = 0; r < rigs_.size(); r++) PS_CUDA(cudaEventRecord(rigs_[r]->slotComputed(rs[r]), comp));

    // ---- copy-out
    PS_CUDA(cudaStreamWaitEvent(sOut_, S.computed, 0));
    for (size_t r = 0; r < rigs_.size(); r++) {
        if (in[r].ydst) {
            const ps_planar_image& d = *in[r].ydst;
            if (d.location != PS_MEM_HOST) continue;
            const uint8_t* out = rigs_[r]->outputBuffer(rs[r]);
            const size_t w = d.width, h = d.height, luma = w * h;
            PS_CUDA(cudaMemcpy2DAsync(d.planes[0], d.pitches[0], out, w, w, h, cudaMemcpyDeviceToHost, sOut_));
            if (d.format == PS_FMT_NV12) {
                PS_CUDA(cudaMemcpy2DAsync(d.planes[1], d.pitches[1], out + luma, w, w, h / 2, cudaMemcpyDeviceToHost,
                                          sOut_));
            } else {
                PS_CUDA(cudaMemcpy2DAsync(d.planes[1], d.pitches[1], out + luma, w / 2, w / 2, h / 2,
                                          cudaMemcpyDeviceToHost, sOut_));
                PS_CUDA(cudaMemcpy2DAsync(d.planes[2], d.pitches[2], out + luma + luma / 4, w / 2, w / 2, h / 2,
                                          cudaMemcpyDeviceToHost, sOut_));
            }
            continue;
        }
        const ps_image& d = *in[r].dst;
        if (d.location == PS_MEM_HOST) {
            const size_t rowBytes = (size_t)d.width * bytesPerPixel(d.format);
            PS_CUDA(cudaMemcpy2DAsync(d.data, d.pitch, rigs_[r]->outputBuffer(rs[r]), rowBytes, rowBytes, d.height,
                                      cudaMemcpyDeviceToHost, sOut_));
        }
    }
    PS_CUDA(cudaEventRecord(S.downloaded, sOut_));
    for (size_t r = 0; r < rigs_.size(); r++) PS_CUDA(cudaEventRecord(rigs_[r]->slotDownloaded(rs[r]), sOut_));
    PS_CUDA(cudaStreamWaitEvent(st, S.downloaded, 0));
    S.used = true;
    nextIo_ = (si + 1) % Rig::kIoSlots;
}

}  // namespace ps
