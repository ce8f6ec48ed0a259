// ps_prepare.cu -- prepare-time kernels: geometry, seams, weight / alpha
// pyramids, tile activity.  Built with --fmad=false so the double-precision
// geometry keeps the reference's separate multiply / add roundings.
#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>

#include "ps_internal.h"

namespace ps {

constexpr double kPi = 3.14159265358979323846264338327950288;
#define PS_DEG_TO_RAD(x) ((x) * 2.0 * kPi / 360.0)

// ============================================================================
// Remap::init (source/Warp/Remap.cpp:147-249) on the host.  The reference
// calls the equirect canvas "src" and the camera frame "dst".
// ============================================================================
static void matMult(const double m1[3][3], const double m2[3][3], double r[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) r[i][k] = m1[i][0] * m2[0][k] + m1[i][1] * m2[1][k] + m1[i][2] * m2[2][k];
}

// SetMatrix, source/Warp/Remap.cpp:22-43
static void setMatrix(double a, double b, double c, double m[3][3], int cl)
{
    double mx[3][3] = {{1.0, 0.0, 0.0}, {0.0, cos(a), sin(a)}, {0.0, 0.0, 0.0}};
    mx[2][1] = -mx[1][2];
    mx[2][2] = mx[1][1];
    double my[3][3] = {{cos(b), 0.0, -sin(b)}, {0.0, 1.0, 0.0}, {0.0, 0.0, 0.0}};
    my[2][0] = -my[0][2];
    my[2][2] = my[0][0];
    double mz[3][3] = {{cos(c), sin(c), 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 1.0}};
    mz[1][0] = -mz[0][1];
    mz[1][1] = mz[0][0];
    double t[3][3];
    if (cl) matMult(mz, mx, t);
    else matMult(mx, mz, t);
    matMult(t, my, m);
}

// smallestRoot and helpers, source/Warp/Remap.cpp:45-135: the smallest
// positive root of the cubic a[3]x^3 + a[2]x^2 + a[1]x + a[0] (1000 if none).
static int polyRoots(const double* a, double* root)
{
    if (a[3] == 0.0) {
        if (a[2] == 0.0) {
            if (a[1] == 0.0) {
                if (a[0] == 0.0) { root[0] = 0.0; return 1; }
                return 0;
            }
            root[0] = -a[0] / a[1];
            return 1;
        }
        if (4.0 * a[2] * a[0] > a[1] * a[1]) return 0;
        root[0] = (-a[1] + sqrt(a[1] * a[1] - 4.0 * a[2] * a[0])) / (2.0 * a[2]);
        root[1] = (-a[1] - sqrt(a[1] * a[1] - 4.0 * a[2] * a[0])) / (2.0 * a[2]);
        return 2;
    }
    const double p = ((-1.0 / 3.0) * (a[2] / a[3]) * (a[2] / a[3]) + a[1] / a[3]) / 3.0;
    const double q = ((2.0 / 27.0) * (a[2] / a[3]) * (a[2] / a[3]) * (a[2] / a[3]) -
                      (1.0 / 3.0) * (a[2] / a[3]) * (a[1] / a[3]) + a[0] / a[3]) / 2.0;
    auto cbrtSigned = [](double x) { return x == 0.0 ? 0.0 : (x > 0.0 ? pow(x, 1.0 / 3.0) : -pow(-x, 1.0 / 3.0)); };
    if (q * q + p * p * p >= 0.0) {
        root[0] = cbrtSigned(-q + sqrt(q * q + p * p * p)) + cbrtSigned(-q - sqrt(q * q + p * p * p)) -
                  a[2] / (3.0 * a[3]);
        return 1;
    }
    const double phi = acos(-q / sqrt(-p * p * p));
    root[0] = 2.0 * sqrt(-p) * cos(phi / 3.0) - a[2] / (3.0 * a[3]);
    root[1] = -2.0 * sqrt(-p) * cos(phi / 3.0 + kPi / 3.0) - a[2] / (3.0 * a[3]);
    root[2] = -2.0 * sqrt(-p) * cos(phi / 3.0 - kPi / 3.0) - a[2] / (3.0 * a[3]);
    return 3;
}

static double smallestPositiveRoot(const double* a)
{
    double root[3], best = 1000.0;
    const int n = polyRoots(a, root);
    for (int i = 0; i < n; i++)
        if (root[i] > 0.0 && root[i] < best) best = root[i];
    return best;
}

void remapInit(const ps_photo_param& param_, int canvasW, int canvasH, int camW, int camH, RemapDev& r)
{
    std::memset(&r, 0, sizeof(r));
    r.srcTX = canvasW / 2;
    r.srcTY = canvasH / 2;
    ps_photo_param p = param_;
    if (p.image_type == 0 || p.image_type == 1) {
        p.crop_x = 0;
        p.crop_y = 0;
        p.crop_width = camW;
        p.crop_height = camH;
    }
    r.type = p.image_type == 0 ? 0 : (p.image_type == 1 ? 3 : 2);
    r.destTX = p.crop_x + p.crop_width / 2;
    r.destTY = p.crop_y + p.crop_height / 2;
    r.horizontal = p.shift_x;
    r.vertical = p.shift_y;
    const double a = PS_DEG_TO_RAD(p.hfov);
    const double b = PS_DEG_TO_RAD(360);
    double mt[3][3];
    setMatrix(-PS_DEG_TO_RAD(p.pitch), 0.0, -PS_DEG_TO_RAD(p.roll), mt, 0);
    for (int i = 0; i < 9; i++) r.mt[i] = mt[i / 3][i % 3];
    r.distance = ((double)canvasW) / b;
    if (r.type == 0) r.scale0 = ((double)p.crop_width) / (2.0 * tan(a / 2.0)) / r.distance;
    else r.scale0 = ((double)p.crop_width) / a / r.distance;
    r.scale1 = r.scale0;
    r.shear0 = p.shear_x / p.crop_height;
    r.shear1 = p.shear_y / p.crop_width;
    r.rot0 = r.distance * kPi;
    r.rot1 = -p.yaw * r.distance * kPi / 180.0;

    double radial[5] = {1.0, 0.0, 0.0, 0.0, 1000.0};
    if (p.beta != 0.0 || p.gamma != 0.0 || p.alpha != 0.0) {
        radial[3] = p.alpha;
        radial[2] = p.beta;
        radial[1] = p.gamma;
        radial[0] = 1.0 - (p.alpha + p.beta + p.gamma);
    }
    double deriv[4];
    for (int k = 0; k < 4; k++) deriv[k] = radial[k] != 0.0 ? (k + 1) * radial[k] : 0.0;
    radial[4] = smallestPositiveRoot(deriv);
    for (int i = 0; i < 4; i++) r.rad[i] = radial[i];
    r.rad[5] = radial[4];
    r.rad[4] = ((double)(p.crop_width < p.crop_height ? p.crop_width : p.crop_height)) / 2.0;

    r.camW = camW;
    r.camH = camH;
    r.circ = (p.image_type == 2 || p.image_type == 3) ? 1 : 0;
    r.cropX = p.crop_x;
    r.cropY = p.crop_y;
    r.cropW = p.crop_width;
    r.cropH = p.crop_height;
    if (r.circ) {
        if (p.circle_r > 0) {
            r.centx = p.circle_x;
            r.centy = p.circle_y;
            r.sqrDist = p.circle_r * p.circle_r;
        } else {
            r.centx = p.crop_x + p.crop_width / 2;
            r.centy = p.crop_y + p.crop_height / 2;
            r.sqrDist = p.crop_width > p.crop_height ? p.crop_width * p.crop_width * 0.25
                                                     : p.crop_height * p.crop_height * 0.25;
        }
    }
}

// getTrueNumLevels, source/Blend/MultiBandBlend.cpp:329-337
int trueNumLevels(int width, int height, int maxLevels, int minLength)
{
    int numLevels = maxLevels < 0 ? 16 : (maxLevels > 16 ? 16 : maxLevels);
    const int side = minLength < 0 ? 2 : (minLength > 64 ? 64 : minLength);
    const int lw = (int)(log((double)width / side) / log(2.0));
    const int lh = (int)(log((double)height / side) / log(2.0));
    const int m = lw < lh ? lw : lh;
    return numLevels < m ? numLevels : m;
}

// ============================================================================
// Remap::remapImage (source/Warp/Remap.cpp:356-514) in double on the GPU,
// the twin of dstToSrc (source/CudaAccel/CudaReproject.cu:81-264).
// ============================================================================
__device__ void rotatedVector(const RemapDev& m, double xs, double ys, double v[3])
{
    xs -= m.srcTX - 0.5;
    ys -= m.srcTY - 0.5;
    double xd = xs + m.rot1;
    while (xd < -m.rot0) xd += 2 * m.rot0;
    while (xd > m.rot0) xd -= 2 * m.rot0;
    double phi = xd / m.distance;
    double theta = -ys / m.distance + kPi / 2;
    if (theta < 0) { theta = -theta; phi += kPi; }
    if (theta > kPi) { theta = kPi - (theta - kPi); phi += kPi; }
    const double v0 = sin(theta) * sin(phi), v1 = cos(theta), v2 = sin(theta) * cos(phi);
    for (int i = 0; i < 3; i++) v[i] = m.mt[0 * 3 + i] * v0 + m.mt[1 * 3 + i] * v1 + m.mt[2 * 3 + i] * v2;
}

__device__ void remapPoint(const RemapDev& m, double cx, double cy, double& ox, double& oy)
{
    double v[3];
    rotatedVector(m, cx, cy, v);
    const double r = sqrt(v[0] * v[0] + v[1] * v[1]);
    const double theta = r == 0.0 ? 0.0 : m.distance * atan2(r, v[2]) / r;
    double x = theta * v[0], y = theta * v[1];
    if (m.type == 0) {
        const double rr = sqrt(x * x + y * y);
        const double th = rr / m.distance;
        const double rho = th >= kPi / 2.0 ? 1.6e16 : (th == 0.0 ? 1.0 : tan(th) / th);
        x = rho * x;
        y = rho * y;
    }
    x = x * m.scale0;
    y = y * m.scale1;
    const double rt = (sqrt(x * x + y * y)) / m.rad[4];
    const double sc = rt < m.rad[5] ? ((m.rad[3] * rt + m.rad[2]) * rt + m.rad[1]) * rt + m.rad[0] : 1000.0;
    x = x * sc;
    y = y * sc;
    if (m.vertical != 0.0) y = y + m.vertical;
    if (m.horizontal != 0.0) x = x + m.horizontal;
    double xd = x, yd = y;
    if (m.shear0 != 0 || m.shear1 != 0) {
        xd = x + m.shear0 * y;
        yd = y + m.shear1 * x;
    }
    ox = xd + (m.destTX - 0.5);
    oy = yd + (m.destTY - 0.5);
}

__device__ __forceinline__ bool mapValid(const RemapDev& m, double sx, double sy)
{
    if (!m.circ) return sx >= 0 && sy >= 0 && sx < m.camW && sy < m.camH;
    return sx >= m.cropX && sy >= m.cropY && sx < m.cropX + m.cropW && sy < m.cropY + m.cropH &&
           (sx - m.centx) * (sx - m.centx) + (sy - m.centy) * (sy - m.centy) < m.sqrDist;
}

// getReprojectMapAndMask + float conversion (source/Warp/ZReproject.cpp:132-240)
__global__ void k_gen_map(const RemapDev* __restrict__ prm, int W, int H, float* xmap, float* ymap, uint8_t* cov)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const RemapDev m = *prm;
    double sx, sy;
    remapPoint(m, x, y, sx, sy);
    const bool ok = mapValid(m, sx, sy);
    const size_t i = (size_t)y * W + x;
    xmap[i] = ok ? (float)sx : -1.f;
    ymap[i] = ok ? (float)sy : -1.f;
    cov[i] = ok ? 255 : 0;
}

cudaError_t launchGenMap(const RemapDev* dParam, int W, int H, float* xmap, float* ymap, uint8_t* cov,
                         cudaStream_t st)
{
    dim3 grid((W + 127) / 128, H);
    k_gen_map<<<grid, 128, 0, st>>>(dParam, W, H, xmap, ymap, cov);
    return cudaGetLastError();
}

// Nearest-optical-axis seams: the covered camera with the smallest angle
// atan2(|v.xy|, v.z) between the pixel ray and its axis (the angle of
// Remap::remapImage, source/Warp/Remap.cpp:416-419); differences under
// 1e-12 rad are ties and go to the lower index.
__global__ void k_seams(const RemapDev* __restrict__ prm, int n, int W, int H, const uint8_t* __restrict__ cov,
                        uint8_t* seams)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const size_t npx = (size_t)W * H, i = (size_t)y * W + x;
    int best = -1;
    double bestA = 0;
    for (int c = 0; c < n; c++) {
        if (!cov[c * npx + i]) continue;
        double v[3];
        rotatedVector(prm[c], x, y, v);
        const double a = atan2(sqrt(v[0] * v[0] + v[1] * v[1]), v[2]);
        if (best < 0 || a < bestA - 1e-12) { best = c; bestA = a; }
    }
    for (int c = 0; c < n; c++) seams[c * npx + i] = c == best ? 255 : 0;
}

cudaError_t launchNearestAxisSeams(const RemapDev* dParams, int n, int W, int H, const uint8_t* cov,
                                   uint8_t* seams, cudaStream_t st)
{
    dim3 grid((W + 127) / 128, H);
    k_seams<<<grid, 128, 0, st>>>(dParams, n, W, H, cov, seams);
    return cudaGetLastError();
}

// ============================================================================
// Reference seams: getNonIntersectingMasks (source/Blend/Mask.cpp:376-398).
// Camera 0 starts with its whole coverage; camera i (i = 1..n-1) takes the
// pixels where the L1 distance to the nearest zero of its own coverage
// exceeds that of the union taken so far, and earlier cameras lose them.
// The L1 distance transform (cv::distanceTransform, CV_DIST_L1, 3x3 mask) is
// computed exactly and separably: the distance along the row to the nearest
// zero (block-wide scans of the last / first zero), then
// d(x, y) = min_y' |y - y'| + r(x, y') by a downward and an upward sweep of
// every column.  Pixels outside the image are not zeros; an image without
// any zero pixel gets kDtFar or more everywhere, above every finite
// distance, which is all the comparisons need.
// ============================================================================
constexpr int kDtFar = 1 << 28;
constexpr int kDtThreads = 256;

__global__ void __launch_bounds__(kDtThreads) k_dt_rows(const uint8_t* __restrict__ mask, int W, int32_t* __restrict__ dist)
{
    __shared__ int sLast[kDtThreads], sFirst[kDtThreads];
    const int t = threadIdx.x;
    const uint8_t* m = mask + (size_t)blockIdx.x * W;
    int32_t* d = dist + (size_t)blockIdx.x * W;
    const int per = (W + kDtThreads - 1) / kDtThreads;
    const int x0 = min(W, t * per), x1 = min(W, x0 + per);
    int last = -1, first = INT_MAX;
    for (int x = x0; x < x1; x++)
        if (!m[x]) {
            if (first == INT_MAX) first = x;
            last = x;
        }
    sLast[t] = last;
    sFirst[t] = first;
    __syncthreads();
    // inclusive prefix max of the last zeros, suffix min of the first zeros
    for (int off = 1; off < kDtThreads; off <<= 1) {
        const int a = t >= off ? sLast[t - off] : -1;
        const int b = t + off < kDtThreads ? sFirst[t + off] : INT_MAX;
        __syncthreads();
        sLast[t] = max(sLast[t], a);
        sFirst[t] = min(sFirst[t], b);
        __syncthreads();
    }
    int L = t > 0 ? sLast[t - 1] : -1;
    for (int x = x0; x < x1; x++) {
        if (!m[x]) L = x;
        d[x] = L < 0 ? kDtFar : x - L;
    }
    int R = t + 1 < kDtThreads ? sFirst[t + 1] : INT_MAX;
    for (int x = x1 - 1; x >= x0; x--) {
        if (!m[x]) R = x;
        if (R != INT_MAX) d[x] = min(d[x], R - x);
    }
}

__global__ void k_dt_cols(int32_t* __restrict__ dist, int W, int H)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    int32_t* c = dist + x;
    int prev = kDtFar;
    for (int y = 0; y < H; y++) {
        const int v = min(c[(size_t)y * W], prev + 1);
        c[(size_t)y * W] = v;
        prev = v;
    }
    prev = kDtFar;
    for (int y = H - 1; y >= 0; y--) {
        const int v = min(c[(size_t)y * W], prev + 1);
        c[(size_t)y * W] = v;
        prev = v;
    }
}

static cudaError_t distanceTransformL1(const uint8_t* mask, int W, int H, int32_t* dist, cudaStream_t st)
{
    k_dt_rows<<<H, kDtThreads, 0, st>>>(mask, W, dist);
    k_dt_cols<<<(W + 127) / 128, 128, 0, st>>>(dist, W, H);
    return cudaGetLastError();
}

__global__ void k_seam_init(const uint8_t* __restrict__ cov, long long total, long long npx, uint8_t* out,
                            uint8_t* uni)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total; p += (long long)gridDim.x * blockDim.x) {
        const uint8_t v = cov[p] ? 255 : 0;
        out[p] = v;
        if (p < npx) uni[p] = v;
    }
}

__global__ void k_seam_take(const int32_t* __restrict__ dCam, const int32_t* __restrict__ dUni, long long npx, int i,
                            uint8_t* out, uint8_t* uni)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        const bool take = dCam[p] > dUni[p];
        out[(size_t)i * npx + p] = take ? 255 : 0;
        if (take) {
            for (int j = 0; j < i; j++) out[(size_t)j * npx + p] = 0;
            uni[p] = 255;
        }
    }
}

cudaError_t launchNonIntersectingMasks(const uint8_t* cov, int n, int W, int H, uint8_t* out, uint8_t* uni,
                                       int32_t* dUni, int32_t* dCam, cudaStream_t st)
{
    const long long npx = (long long)W * H;
    const int grid = (int)std::min<long long>((npx * n + 255) / 256, 4096);
    k_seam_init<<<grid, 256, 0, st>>>(cov, npx * n, npx, out, uni);
    cudaError_t e = cudaGetLastError();
    for (int i = 1; i < n && e == cudaSuccess; i++) {
        e = distanceTransformL1(uni, W, H, dUni, st);
        if (e == cudaSuccess) e = distanceTransformL1(out + (size_t)i * npx, W, H, dCam, st);
        if (e == cudaSuccess) {
            k_seam_take<<<(int)std::min<long long>((npx + 255) / 256, 4096), 256, 0, st>>>(dCam, dUni, npx, i, out,
                                                                                          uni);
            e = cudaGetLastError();
        }
    }
    return e;
}

// Standalone distance transform (tests and callers of the primitive).
cudaError_t launchDistanceTransformL1(const uint8_t* mask, int W, int H, int32_t* dist, cudaStream_t st)
{
    return distanceTransformL1(mask, W, H, dist, st);
}

// ============================================================================
// Weight and alpha pyramids (CudaTilingMultibandBlendFast::prepare,
// source/CudaAccel/CudaMultibandBlend.cpp:586-605), one thread per output.
// ============================================================================
__global__ void k_init_level0(const uint8_t* __restrict__ cov, const uint8_t* __restrict__ seams, int W, int H,
                              long long maskStride, uint16_t* wt, uint16_t* a0, int pitch, long long camStride)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= W) return;
    const size_t mi = (size_t)c * maskStride + (size_t)y * W + x;
    const size_t o = (size_t)c * camStride + (size_t)y * pitch + x;
    wt[o] = seams[mi] ? 256 : 0;
    a0[o] = cov[mi] ? 256 : 0;
}

cudaError_t launchInitLevel0(const uint8_t* cov, const uint8_t* seams, int W, int H, long long maskStride,
                             uint16_t* wt, uint16_t* a0, int pitch, long long camStride, int n, cudaStream_t st)
{
    dim3 grid((W + 127) / 128, H, n);
    k_init_level0<<<grid, 128, 0, st>>>(cov, seams, W, H, maskStride, wt, a0, pitch, camStride);
    return cudaGetLastError();
}

__device__ __forceinline__ int downSum16(const uint16_t* s, int sw, int sh, int spitch, int x, int y)
{
    const int k5[5] = {1, 4, 6, 4, 1};
    int sum = 0;
    for (int dy = 0; dy < 5; dy++) {
        const uint16_t* row = s + (size_t)rowMap(2 * y + dy - 2, sh) * spitch;
        int rs = 0;
        for (int dx = 0; dx < 5; dx++) rs += k5[dx] * (int)row[colMap(2 * x + dx - 2, sw)];
        sum += k5[dy] * rs;
    }
    return sum;
}

// pyrDown16SC1To32SC1 (CudaPyramid2.cu:16-122) + scaledSet16SC1Mask32SC1 (:804-813)
__global__ void k_alpha_down(const uint16_t* __restrict__ aj, int sw, int sh, int spitch, long long sstride,
                             uint16_t* am, uint16_t* anext, int dw, int dh, int dpitch, long long dstride)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= dw) return;
    const int s = downSum16(aj + c * sstride, sw, sh, spitch, x, y);
    const size_t o = (size_t)c * dstride + (size_t)y * dpitch + x;
    am[o] = (uint16_t)(s >> 8);
    anext[o] = s ? 256 : 0;
}

cudaError_t launchAlphaDown(const uint16_t* aj, int sw, int sh, int spitch, long long sstride, uint16_t* am,
                            uint16_t* anext, int dw, int dh, int dpitch, long long dstride, int n, cudaStream_t st)
{
    dim3 grid((dw + 127) / 128, dh, n);
    k_alpha_down<<<grid, 128, 0, st>>>(aj, sw, sh, spitch, sstride, am, anext, dw, dh, dpitch, dstride);
    return cudaGetLastError();
}

// pyrDown16SC1To16SC1 (CudaPyramid2.cu:124-226): (S + 128) >> 8
__global__ void k_weight_down(const uint16_t* __restrict__ wj, int sw, int sh, int spitch, long long sstride,
                              uint16_t* wn, int dw, int dh, int dpitch, long long dstride)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= dw) return;
    const int s = downSum16(wj + c * sstride, sw, sh, spitch, x, y);
    wn[(size_t)c * dstride + (size_t)y * dpitch + x] = (uint16_t)((s + 128) >> 8);
}

cudaError_t launchWeightDown(const uint16_t* wj, int sw, int sh, int spitch, long long sstride, uint16_t* wn,
                             int dw, int dh, int dpitch, long long dstride, int n, cudaStream_t st)
{
    dim3 grid((dw + 127) / 128, dh, n);
    k_weight_down<<<grid, 128, 0, st>>>(wj, sw, sh, spitch, sstride, wn, dw, dh, dpitch, dstride);
    return cudaGetLastError();
}

// ============================================================================
// Tile activity
// ============================================================================
template <class T>
__global__ void k_tile_flags(const T* __restrict__ p, int w, int h, int pitch, long long camStride, int tw, int th,
                             int tilesX, int tilesY, uint8_t* flags)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= w) return;
    if (p[(size_t)c * camStride + (size_t)y * pitch + x] != 0)
        flags[((size_t)c * tilesY + y / th) * tilesX + x / tw] = 1;
}

cudaError_t launchTileFlags16(const uint16_t* p, int w, int h, int pitch, long long camStride, int n, int tw,
                              int th, int tilesX, int tilesY, uint8_t* flags, cudaStream_t st)
{
    dim3 grid((w + 127) / 128, h, n);
    k_tile_flags<uint16_t><<<grid, 128, 0, st>>>(p, w, h, pitch, camStride, tw, th, tilesX, tilesY, flags);
    return cudaGetLastError();
}

// per-tile "some pixel differs from 256" flags of a weight plane
__global__ void k_tile_not256(const uint16_t* __restrict__ p, int w, int h, int pitch, long long camStride, int tw,
                              int th, int tilesX, int tilesY, uint8_t* flags)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= w) return;
    if (p[(size_t)c * camStride + (size_t)y * pitch + x] != 256)
        flags[((size_t)c * tilesY + y / th) * tilesX + x / tw] = 1;
}

cudaError_t launchTileNot256(const uint16_t* p, int w, int h, int pitch, long long camStride, int n, int tw, int th,
                             int tilesX, int tilesY, uint8_t* flags, cudaStream_t st)
{
    dim3 grid((w + 127) / 128, h, n);
    k_tile_not256<<<grid, 128, 0, st>>>(p, w, h, pitch, camStride, tw, th, tilesX, tilesY, flags);
    return cudaGetLastError();
}

cudaError_t launchTileFlags8(const uint8_t* p, int w, int h, int pitch, long long camStride, int n, int tw,
                             int th, int tilesX, int tilesY, uint8_t* flags, cudaStream_t st)
{
    dim3 grid((w + 127) / 128, h, n);
    k_tile_flags<uint8_t><<<grid, 128, 0, st>>>(p, w, h, pitch, camStride, tw, th, tilesX, tilesY, flags);
    return cudaGetLastError();
}

// number of non-zero pixels of a 16-bit plane over all cameras
__global__ void k_count_nonzero16(const uint16_t* __restrict__ p, int w, int h, int pitch, long long camStride,
                                  unsigned long long* out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    const int nz = x < w && p[(size_t)c * camStride + (size_t)y * pitch + x] != 0;
    const int cnt = __syncthreads_count(nz);
    if (threadIdx.x == 0 && cnt) atomicAdd(out, (unsigned long long)cnt);
}

cudaError_t launchCountNonzero16(const uint16_t* p, int w, int h, int pitch, long long camStride, int n,
                                 unsigned long long* out, cudaStream_t st)
{
    dim3 grid((w + 127) / 128, h, n);
    k_count_nonzero16<<<grid, 128, 0, st>>>(p, w, h, pitch, camStride, out);
    return cudaGetLastError();
}

// union coverage; one block of tw x th threads per tile counts covered pixels
__global__ void k_union(const uint8_t* __restrict__ cov, int n, int W, int H, long long maskStride, uint8_t* uni,
                        int pitch, int tilesX, int* tileCounts, unsigned long long* total)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    int covered = 0;
    if (x < W && y < H) {
        for (int c = 0; c < n && !covered; c++) covered = cov[(size_t)c * maskStride + (size_t)y * W + x] != 0;
        uni[(size_t)y * pitch + x] = covered ? 255 : 0;
    }
    const int cnt = __syncthreads_count(covered);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        tileCounts[blockIdx.y * tilesX + blockIdx.x] = cnt;
        atomicAdd(total, (unsigned long long)cnt);
    }
}

cudaError_t launchUnion(const uint8_t* cov, int n, int W, int H, long long maskStride, uint8_t* uni, int pitch,
                        int tw, int th, int tilesX, int* tileCounts, unsigned long long* total, cudaStream_t st)
{
    dim3 block(tw, th);
    dim3 grid((W + tw - 1) / tw, (H + th - 1) / th);
    k_union<<<grid, block, 0, st>>>(cov, n, W, H, maskStride, uni, pitch, tilesX, tileCounts, total);
    return cudaGetLastError();
}

__global__ void k_compact_maps(const float* __restrict__ xmap, const float* __restrict__ ymap, int W, int H,
                               long long maskStride, const RemapItem* __restrict__ items, float2* maps)
{
    const RemapItem it = items[blockIdx.x];
    const int x = it.tx * kRemapTW + (threadIdx.x & 31), y = it.ty * kRemapTH + (threadIdx.x >> 5);
    float2 v = make_float2(-1.f, -1.f);
    if (x < W && y < H) {
        const size_t i = (size_t)it.cam * maskStride + (size_t)y * W + x;
        v = make_float2(xmap[i], ymap[i]);
    }
    maps[(size_t)it.mapTile * (kRemapTW * kRemapTH) + threadIdx.x] = v;
}

// Coverage of each remap tile as 16 words (one per tile row, bit = column),
// for the map-free remap: one warp per row, one ballot per word.
__global__ void k_cov_tiles(const uint8_t* __restrict__ cov, int W, int H, long long maskStride,
                            const RemapItem* __restrict__ items, uint32_t* words)
{
    const RemapItem it = items[blockIdx.x];
    const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
    const int x = it.tx * kRemapTW + lx, y = it.ty * kRemapTH + ly;
    const bool c = x < W && y < H && cov[(size_t)it.cam * maskStride + (size_t)y * W + x] != 0;
    const uint32_t w = __ballot_sync(0xffffffffu, c);
    if (lx == 0) words[(size_t)it.mapTile * kRemapTH + ly] = w;
}

cudaError_t launchCovTiles(const uint8_t* cov, int W, int H, long long maskStride, const RemapItem* items,
                           int nitems, uint32_t* words, cudaStream_t st)
{
    if (nitems <= 0) return cudaSuccess;
    k_cov_tiles<<<nitems, kRemapTW * kRemapTH, 0, st>>>(cov, W, H, maskStride, items, words);
    return cudaGetLastError();
}

RemapParamF remapParamF(const RemapDev& r)
{
    RemapParamF f;
    f.type = r.type;
    f.srcTX = (float)r.srcTX;
    f.srcTY = (float)r.srcTY;
    f.destTX = (float)r.destTX;
    f.destTY = (float)r.destTY;
    f.scale0 = (float)r.scale0;
    f.scale1 = (float)r.scale1;
    f.shear0 = (float)r.shear0;
    f.shear1 = (float)r.shear1;
    f.rot0 = (float)r.rot0;
    f.rot1 = (float)r.rot1;
    for (int i = 0; i < 6; i++) f.rad[i] = (float)r.rad[i];
    for (int i = 0; i < 9; i++) f.mt[i] = (float)r.mt[i];
    f.distance = (float)r.distance;
    f.horizontal = (float)r.horizontal;
    f.vertical = (float)r.vertical;
    return f;
}

cudaError_t launchCompactMaps(const float* xmap, const float* ymap, int W, int H, long long maskStride,
                              const RemapItem* items, int nitems, float2* maps, cudaStream_t st)
{
    if (nitems <= 0) return cudaSuccess;
    k_compact_maps<<<nitems, kRemapTW * kRemapTH, 0, st>>>(xmap, ymap, W, H, maskStride, items, maps);
    return cudaGetLastError();
}

// ============================================================================
// Linear-blend weights: getWeightsLinearBlend32F (source/Blend/LinearBlend.cpp:
// 136-151) and calcWeights32F (:78-120).  Per camera, the 0/255 seam mask is
// blurred by a (2r+1)-tap Gaussian (sigma r/3) with cv::GaussianBlur's
// default reflect-101 border, in 8-bit fixed point (row and column taps
// scaled by 2^8, the 2^16-scaled sum rounded and saturated), ANDed with the
// 0/255 coverage; at each pixel the blurred values then become weights:
// d_k / sum_k d_k (fp32, one reciprocal, one product) where two or more
// cameras are non-zero, 1 where exactly one is.
// ============================================================================
// reflect-101 index with repeated reflection (cv::borderInterpolate)
__device__ __forceinline__ int reflect101(int p, int len)
{
    if (len == 1) return 0;
    while (p < 0 || p >= len) p = p < 0 ? -p : 2 * len - 2 - p;
    return p;
}

// grid (H, n): one CTA per row of one camera; the row is staged with its
// reflected borders in shared memory (W + 2r bytes).
__global__ void k_gauss_rows(const uint8_t* __restrict__ seam, int W, int H, const int* __restrict__ taps, int r,
                             int32_t* __restrict__ rows)
{
    extern __shared__ uint8_t ext[];
    const int y = blockIdx.x, c = blockIdx.y;
    const uint8_t* src = seam + ((size_t)c * H + y) * W;
    for (int k = threadIdx.x; k < W + 2 * r; k += blockDim.x) ext[k] = src[reflect101(k - r, W)] ? 255 : 0;
    __syncthreads();
    int32_t* out = rows + ((size_t)c * H + y) * W;
    for (int x = threadIdx.x; x < W; x += blockDim.x) {
        int acc = 0;
        for (int k = 0; k <= 2 * r; k++) acc += __ldg(taps + k) * ext[x + k];
        out[x] = acc;
    }
}

// grid (ceil(W / 128), H, n): the column pass, rounding, saturation and the
// AND with the coverage.
__global__ void k_gauss_cols(const int32_t* __restrict__ rows, const uint8_t* __restrict__ cov, int W, int H,
                             const int* __restrict__ taps, int r, uint8_t* __restrict__ dist)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= W) return;
    const int32_t* col = rows + (size_t)c * H * W + x;
    long long acc = 0;
    for (int k = 0; k <= 2 * r; k++) acc += (long long)__ldg(taps + k) * col[(size_t)reflect101(y + k - r, H) * W];
    const long long v = (acc + (1 << 15)) >> 16;
    const size_t o = ((size_t)c * H + y) * W + x;
    dist[o] = cov[o] ? (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)) : 0;
}

__global__ void k_linear_weights(const uint8_t* __restrict__ dist, int n, long long npx, float* __restrict__ w)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
        float sum = 0.f;
        int count = 0, last = 0;
        for (int k = 0; k < n; k++) {
            const int d = dist[(size_t)k * npx + p];
            sum = __fadd_rn(sum, (float)d);
            if (d) {
                count++;
                last = k;
            }
        }
        const float inv = count > 1 ? __fdiv_rn(1.f, sum) : 0.f;
        for (int k = 0; k < n; k++) {
            float v = 0.f;
            if (count > 1) v = __fmul_rn((float)dist[(size_t)k * npx + p], inv);
            else if (count == 1 && k == last) v = 1.f;
            w[(size_t)k * npx + p] = v;
        }
    }
}

__global__ void k_compact_weights(const float* __restrict__ w, int W, int H, long long npx,
                                  const RemapItem* __restrict__ items, float* out)
{
    const RemapItem it = items[blockIdx.x];
    const int x = it.tx * kRemapTW + (threadIdx.x & 31), y = it.ty * kRemapTH + (threadIdx.x >> 5);
    out[(size_t)it.mapTile * (kRemapTW * kRemapTH) + threadIdx.x] =
        (x < W && y < H) ? w[(size_t)it.cam * npx + (size_t)y * W + x] : 0.f;
}

cudaError_t launchLinearWeights(const uint8_t* seam, const uint8_t* cov, int n, int W, int H, const int* taps, int r,
                                int32_t* rowsScratch, uint8_t* distScratch, float* wFull, const RemapItem* items,
                                int nitems, float* wCompact, cudaStream_t st)
{
    const long long npx = (long long)W * H;
    k_gauss_rows<<<dim3(H, n), 256, W + 2 * r, st>>>(seam, W, H, taps, r, rowsScratch);
    k_gauss_cols<<<dim3((W + 127) / 128, H, n), 128, 0, st>>>(rowsScratch, cov, W, H, taps, r, distScratch);
    k_linear_weights<<<(int)std::min<long long>((npx + 255) / 256, 8192), 256, 0, st>>>(distScratch, n, npx, wFull);
    if (nitems > 0) k_compact_weights<<<nitems, kRemapTW * kRemapTH, 0, st>>>(wFull, W, H, npx, items, wCompact);
    return cudaGetLastError();
}

// Blender input images -> uchar4 level 0.  status bit 1: a 16-bit value
// outside 0..255; bit 2: a non-zero pixel where the coverage mask is 0 (the
// multiband blend needs zeros there, source/Warp/ZReproject.cpp:200-208).
__global__ void k_images_to_level0(const void* const* __restrict__ images, const long long* __restrict__ pitches,
                                   int fmt, int W, int H, const uint8_t* __restrict__ cov, long long maskStride,
                                   uchar4* g0, int pitch, long long camStride, int* status)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= W) return;
    const uint8_t* row = static_cast<const uint8_t*>(images[c]) + (size_t)y * pitches[c];
    int b, g, r;
    if (fmt == 16) {
        const short4 v = reinterpret_cast<const short4*>(row)[x];
        b = v.x; g = v.y; r = v.z;
        if ((unsigned)b > 255u || (unsigned)g > 255u || (unsigned)r > 255u) {
            atomicOr(status, 1);
            b = min(max(b, 0), 255); g = min(max(g, 0), 255); r = min(max(r, 0), 255);
        }
    } else {
        const uchar4 v = reinterpret_cast<const uchar4*>(row)[x];
        b = v.x; g = v.y; r = v.z;
    }
    if (!cov[(size_t)c * maskStride + (size_t)y * W + x] && (b | g | r)) atomicOr(status, 2);
    g0[(size_t)c * camStride + (size_t)y * pitch + x] = make_uchar4(b, g, r, 0);
}

cudaError_t launchImagesToLevel0(const void* const* images, const long long* pitches, int fmt, int n, int W, int H,
                                 const uint8_t* cov, long long maskStride, uchar4* g0, int pitch,
                                 long long camStride, int* status, cudaStream_t st)
{
    dim3 grid((W + 127) / 128, H, n);
    k_images_to_level0<<<grid, 128, 0, st>>>(images, pitches, fmt, W, H, cov, maskStride, g0, pitch, camStride,
                                             status);
    return cudaGetLastError();
}

}  // namespace ps

// ============================================================================
// Allocation-free seam masks.
//
// Some callers cannot call cudaMalloc: a host that has handed its device
// memory budget to another allocator and must not touch the driver's heap,
// a real-time thread where an allocation (which may synchronise the device)
// would blow the frame deadline, or code that must run while other work on
// the device cannot be disturbed.  For them this entry point computes the
// nearest-optical-axis seam masks (what ps_render_prepare does internally)
// with all of its scratch -- the cameras' parameters and coverage masks -- in
// one fixed array that lives in the library image.  The array holds
// kNoAllocScratchBytes on every GPU that loads the library, until the
// process exits.
// ============================================================================
namespace ps {
namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB
constexpr size_t kNoAllocParamBytes = 64 * 1024;    // camera parameters at the front
static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

// Device address of g_noallocScratch per device, looked up once per device.
std::mutex g_noallocMu;
void* g_noallocPtr[64] = {};

}  // namespace

// The cameras' parameters travel to the device as the argument of a kernel
// (by value, copied at launch), which writes them into the scratch array:
// no host buffer is read after the call returns and no copy waits on the
// host.  64 cameras x 288 bytes stay inside the 32 KB argument limit.
struct NoAllocParams {
    RemapDev cam[PS_MAX_CAMS];
};
static_assert(sizeof(NoAllocParams) <= 32000, "camera parameters exceed the kernel argument limit");

__global__ void k_noalloc_params(const __grid_constant__ NoAllocParams p, int n, RemapDev* out)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = p.cam[i];
}

// coverage only (getReprojectMapAndMask's mask), as k_gen_map computes it
__global__ void k_coverage(const RemapDev* __restrict__ prm, int W, int H, uint8_t* cov)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, c = blockIdx.z;
    if (x >= W) return;
    const RemapDev m = prm[c];
    double sx, sy;
    remapPoint(m, x, y, sx, sy);
    cov[(size_t)c * W * H + (size_t)y * W + x] = mapValid(m, sx, sy) ? 255 : 0;
}

}  // namespace ps

extern "C" int ps_nearest_axis_seams_no_alloc(const ps_photo_param* params, int num_params, int src_w, int src_h,
                                              int dst_w, int dst_h, uint8_t* seams, void* stream)
{
    using namespace ps;
    try {
        if (!params || !seams || num_params <= 0) fail(PS_EINVAL, "NULL argument or no cameras");
        if (num_params > PS_MAX_CAMS) fail(PS_EINVAL, "%d cameras, at most %d supported", num_params, PS_MAX_CAMS);
        if (src_w <= 0 || src_h <= 0 || dst_w <= 0 || dst_h <= 0) fail(PS_EINVAL, "sizes must be positive");
        if (dst_h > 65535) fail(PS_EINVAL, "dst_h %d exceeds 65535 (one grid row per canvas row)", dst_h);
        for (int i = 0; i < num_params; i++)
            if (params[i].image_type < 0 || params[i].image_type > 3)
                fail(PS_EINVAL, "camera %d: image_type %d not in 0..3", i, params[i].image_type);
        const size_t covBytes = (size_t)num_params * dst_w * dst_h;
        if (covBytes > kNoAllocScratchBytes - kNoAllocParamBytes)
            fail(PS_EINVAL,
                 "%d cameras x %d x %d coverage bytes exceed the %zu-byte scratch of the allocation-free path "
                 "(use ps_render_prepare)",
                 num_params, dst_w, dst_h, kNoAllocScratchBytes - kNoAllocParamBytes);
        int dev = 0;
        PS_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64) fail(PS_EINVAL, "device %d out of range", dev);
        void* base = nullptr;
        {
            std::lock_guard<std::mutex> lk(g_noallocMu);
            if (!g_noallocPtr[dev]) {
                // the symbol's device address on the current device (the host-side
                // name is only a stand-in and must never reach a kernel)
                PS_CUDA(cudaGetSymbolAddress(&g_noallocPtr[dev], g_noallocScratch));
            }
            base = g_noallocPtr[dev];
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        RemapDev* dParams = static_cast<RemapDev*>(base);
        uint8_t* cov = static_cast<uint8_t*>(base) + kNoAllocParamBytes;
        static_assert(sizeof(RemapDev) * PS_MAX_CAMS <= kNoAllocParamBytes, "parameter area too small");
        NoAllocParams rp;
        for (int i = 0; i < num_params; i++) remapInit(params[i], dst_w, dst_h, src_w, src_h, rp.cam[i]);
        k_noalloc_params<<<1, 64, 0, st>>>(rp, num_params, dParams);
        PS_CUDA(cudaGetLastError());
        // every coverage byte is rewritten, so nothing of the last call's contents survives
        dim3 grid((dst_w + 127) / 128, dst_h, num_params);
        k_coverage<<<grid, 128, 0, st>>>(dParams, dst_w, dst_h, cov);
        PS_CUDA(cudaGetLastError());
        PS_CUDA(launchNearestAxisSeams(dParams, num_params, dst_w, dst_h, cov, seams, st));
        return PS_OK;
    } catch (const Error& e) {
        setLastError(e.what());
        return e.code;
    } catch (const std::exception& e) {
        setLastError(e.what());
        return PS_EINVAL;
    }
}
