/*
 * ps_oracle.c -- CPU restatement of PanoStitcher's per-frame stitch path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA product path and the
 * timed CPU baseline.  Nothing in panostitcher_gb300/ links or calls it.
 * Parity is pinned against the reference's own code built in oracle/_ref/;
 * see ps_oracle.h.
 *
 * Compile with -ffp-contract=off: the double-precision remap and geometry
 * must not be fused into FMAs, so that x86-64 and aarch64 builds agree.
 */
#include "ps_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================== */
/* Geometry: source/Warp/Remap.cpp                                           */
/* ======================================================================== */

static const double ORC_PI = 3.14159265358979323846264338327950288;
#define ORC_DEG_TO_RAD(x) ((x) * 2.0 * ORC_PI / 360.0)

/* matrix_matrix_mult, source/Warp/Remap.cpp:9-20 */
static void mat_mult(double m1[3][3], double m2[3][3], double result[3][3])
{
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            result[i][k] = m1[i][0] * m2[0][k] + m1[i][1] * m2[1][k] + m1[i][2] * m2[2][k];
}

/* SetMatrix, source/Warp/Remap.cpp:22-43 */
static void set_matrix(double a, double b, double c, double m[3][3], int cl)
{
    double mx[3][3], my[3][3], mz[3][3], tmp[3][3];
    mx[0][0] = 1.0; mx[0][1] = 0.0;     mx[0][2] = 0.0;
    mx[1][0] = 0.0; mx[1][1] = cos(a);  mx[1][2] = sin(a);
    mx[2][0] = 0.0; mx[2][1] = -mx[1][2]; mx[2][2] = mx[1][1];

    my[0][0] = cos(b); my[0][1] = 0.0; my[0][2] = -sin(b);
    my[1][0] = 0.0;    my[1][1] = 1.0; my[1][2] = 0.0;
    my[2][0] = -my[0][2]; my[2][1] = 0.0; my[2][2] = my[0][0];

    mz[0][0] = cos(c);     mz[0][1] = sin(c);    mz[0][2] = 0.0;
    mz[1][0] = -mz[0][1];  mz[1][1] = mz[0][0];  mz[1][2] = 0.0;
    mz[2][0] = 0.0;        mz[2][1] = 0.0;       mz[2][2] = 1.0;

    if (cl) mat_mult(mz, mx, tmp);
    else    mat_mult(mx, mz, tmp);
    mat_mult(tmp, my, m);
}

/* squareZero / cubeRoot / cubeZero / smallestRoot, source/Warp/Remap.cpp:45-135 */
static void square_zero(double* a, int* n, double* root)
{
    if (a[2] == 0.0) {
        if (a[1] == 0.0) {
            if (a[0] == 0.0) { *n = 1; root[0] = 0.0; }
            else *n = 0;
        } else { *n = 1; root[0] = -a[0] / a[1]; }
    } else {
        if (4.0 * a[2] * a[0] > a[1] * a[1]) *n = 0;
        else {
            *n = 2;
            root[0] = (-a[1] + sqrt(a[1] * a[1] - 4.0 * a[2] * a[0])) / (2.0 * a[2]);
            root[1] = (-a[1] - sqrt(a[1] * a[1] - 4.0 * a[2] * a[0])) / (2.0 * a[2]);
        }
    }
}

static double cube_root(double x)
{
    if (x == 0.0) return 0.0;
    if (x > 0.0) return pow(x, 1.0 / 3.0);
    return -pow(-x, 1.0 / 3.0);
}

static void cube_zero(double* a, int* n, double* root)
{
    if (a[3] == 0.0) { square_zero(a, n, root); return; }
    double p = ((-1.0 / 3.0) * (a[2] / a[3]) * (a[2] / a[3]) + a[1] / a[3]) / 3.0;
    double q = ((2.0 / 27.0) * (a[2] / a[3]) * (a[2] / a[3]) * (a[2] / a[3]) -
                (1.0 / 3.0) * (a[2] / a[3]) * (a[1] / a[3]) + a[0] / a[3]) / 2.0;
    if (q * q + p * p * p >= 0.0) {
        *n = 1;
        root[0] = cube_root(-q + sqrt(q * q + p * p * p)) + cube_root(-q - sqrt(q * q + p * p * p)) -
                  a[2] / (3.0 * a[3]);
    } else {
        double phi = acos(-q / sqrt(-p * p * p));
        *n = 3;
        root[0] = 2.0 * sqrt(-p) * cos(phi / 3.0) - a[2] / (3.0 * a[3]);
        root[1] = -2.0 * sqrt(-p) * cos(phi / 3.0 + ORC_PI / 3.0) - a[2] / (3.0 * a[3]);
        root[2] = -2.0 * sqrt(-p) * cos(phi / 3.0 - ORC_PI / 3.0) - a[2] / (3.0 * a[3]);
    }
}

static double smallest_root(double* p)
{
    int n = 0;
    double root[3], sroot = 1000.0;
    cube_zero(p, &n, root);
    for (int i = 0; i < n; i++)
        if (root[i] > 0.0 && root[i] < sroot) sroot = root[i];
    return sroot;
}

/* Remap::init, source/Warp/Remap.cpp:147-249.  The reference names the
   equirect canvas "src" and the camera image "dst"; here the arguments are
   named for what they are. */
void orc_remap_init(const orc_param* param_, int canvasW, int canvasH, int camW, int camH, orc_remap* r)
{
    memset(r, 0, sizeof(*r));
    r->srcTX = canvasW / 2;
    r->srcTY = canvasH / 2;

    orc_param param = *param_;
    int fullImage = param.imageType == 0 || param.imageType == 1;
    if (fullImage) {
        param.cropX = 0;
        param.cropY = 0;
        param.cropWidth = camW;
        param.cropHeight = camH;
    }
    if (param.imageType == 0) r->srcImageType = 0;        /* PTImageTypeRectlinear */
    else if (param.imageType == 1) r->srcImageType = 3;   /* PTImageTypeFullFrameFishEye */
    else r->srcImageType = 2;                             /* PTImageTypeCircularFishEye */

    r->destTX = param.cropX + param.cropWidth / 2;
    r->destTY = param.cropY + param.cropHeight / 2;
    r->horizontal = param.shiftX != 0 ? param.shiftX : 0;
    r->vertical = param.shiftY != 0 ? param.shiftY : 0;

    double a = ORC_DEG_TO_RAD(param.hfov);
    double b = ORC_DEG_TO_RAD(360);
    set_matrix(-ORC_DEG_TO_RAD(param.pitch), 0.0, -ORC_DEG_TO_RAD(param.roll), r->mt, 0);
    r->distance = ((double)canvasW) / b;
    if (r->srcImageType == 0)
        r->scale[0] = ((double)param.cropWidth) / (2.0 * tan(a / 2.0)) / r->distance;
    else
        r->scale[0] = ((double)param.cropWidth) / a / r->distance;
    r->scale[1] = r->scale[0];
    r->shear[0] = param.shearX / param.cropHeight;
    r->shear[1] = param.shearY / param.cropWidth;
    r->rot[0] = r->distance * ORC_PI;
    r->rot[1] = -param.yaw * r->distance * ORC_PI / 180.0;

    double radial[3][5];
    for (int i = 0; i < 3; i++) {
        radial[i][0] = 1.0;
        radial[i][4] = 1000.0;
        for (int k = 1; k < 4; k++) radial[i][k] = 0.0;
    }
    if (param.beta != 0.0 || param.gamma != 0.0 || param.alpha != 0.0) {
        for (int i = 0; i < 3; i++) {
            radial[i][3] = param.alpha;
            radial[i][2] = param.beta;
            radial[i][1] = param.gamma;
            radial[i][0] = 1.0 - (param.alpha + param.beta + param.gamma);
        }
    }
    double temp[4];
    for (int i = 0; i < 3; i++) {
        for (int k = 0; k < 4; k++) {
            temp[k] = 0.0;
            if (radial[i][k] != 0.0) temp[k] = (k + 1) * radial[i][k];
        }
        radial[i][4] = smallest_root(temp);
    }
    for (int i = 0; i < 4; i++) r->rad[i] = radial[0][i];
    r->rad[5] = radial[0][4];
    r->rad[4] = ((double)(param.cropWidth < param.cropHeight ? param.cropWidth : param.cropHeight)) / 2.0;
}

/* Remap::remapImage up to the rotated unit vector, source/Warp/Remap.cpp:356-407 */
static void remap_rotated_vector(const orc_remap* m, double x_src, double y_src, double v[3])
{
    double x_dest;
    x_src -= m->srcTX - 0.5;
    y_src -= m->srcTY - 0.5;
    x_dest = x_src + m->rot[1];
    while (x_dest < -m->rot[0]) x_dest += 2 * m->rot[0];
    while (x_dest > m->rot[0]) x_dest -= 2 * m->rot[0];
    x_src = x_dest;

    double phi = x_src / m->distance;
    double theta = -y_src / m->distance + ORC_PI / 2;
    if (theta < 0) { theta = -theta; phi += ORC_PI; }
    if (theta > ORC_PI) { theta = ORC_PI - (theta - ORC_PI); phi += ORC_PI; }
    double v0 = sin(theta) * sin(phi);
    double v1 = cos(theta);
    double v2 = sin(theta) * cos(phi);
    for (int i = 0; i < 3; i++)
        v[i] = m->mt[0][i] * v0 + m->mt[1][i] * v1 + m->mt[2][i] * v2;
}

/* Remap::remapImage, source/Warp/Remap.cpp:356-514 */
void orc_remap_point(const orc_remap* m, double cx, double cy, double* out_x, double* out_y)
{
    double v[3];
    remap_rotated_vector(m, cx, cy, v);
    double r = sqrt(v[0] * v[0] + v[1] * v[1]);
    double theta;
    if (r == 0.0) theta = 0.0;
    else theta = m->distance * atan2(r, v[2]) / r;
    double x_src = theta * v[0];
    double y_src = theta * v[1];

    if (m->srcImageType == 0) {
        double rr = sqrt(x_src * x_src + y_src * y_src);
        double th = rr / m->distance;
        double rho;
        if (th >= ORC_PI / 2.0) rho = 1.6e16;
        else if (th == 0.0) rho = 1.0;
        else rho = tan(th) / th;
        x_src = rho * x_src;
        y_src = rho * y_src;
    }
    x_src = x_src * m->scale[0];
    y_src = y_src * m->scale[1];

    double rt = (sqrt(x_src * x_src + y_src * y_src)) / m->rad[4];
    double sc;
    if (rt < m->rad[5]) sc = ((m->rad[3] * rt + m->rad[2]) * rt + m->rad[1]) * rt + m->rad[0];
    else sc = 1000.0;
    x_src = x_src * sc;
    y_src = y_src * sc;

    if (m->vertical != 0.0) y_src = y_src + m->vertical;
    if (m->horizontal != 0.0) x_src = x_src + m->horizontal;
    double x_dest = x_src, y_dest = y_src;
    if (m->shear[0] != 0 || m->shear[1] != 0) {
        x_dest = x_src + m->shear[0] * y_src;
        y_dest = y_src + m->shear[1] * x_src;
    }
    x_dest += m->destTX - 0.5;
    y_dest += m->destTY - 0.5;
    *out_x = x_dest;
    *out_y = y_dest;
}

/* Angle between the canvas pixel's ray and the camera's optical axis: the
   atan2(r, v[2]) of Remap::remapImage (source/Warp/Remap.cpp:416-419). */
double orc_remap_axis_angle(const orc_remap* m, double cx, double cy)
{
    double v[3];
    remap_rotated_vector(m, cx, cy, v);
    return atan2(sqrt(v[0] * v[0] + v[1] * v[1]), v[2]);
}

/* getReprojectMapAndMask (source/Warp/ZReproject.cpp:132-219) followed by
   the float conversion of getReprojectMap32FAndMask (:231-240). */
void orc_reproject_map(const orc_param* p, int camW, int camH, int canvasW, int canvasH,
                       double* map64, float* xmap, float* ymap, uint8_t* mask)
{
    orc_reproject_map_rows(p, camW, camH, canvasW, canvasH, 0, canvasH, map64, xmap, ymap, mask);
}

void orc_reproject_map_rows(const orc_param* p, int camW, int camH, int canvasW, int canvasH, int row0, int row1,
                            double* map64, float* xmap, float* ymap, uint8_t* mask)
{
    orc_remap m;
    orc_remap_init(p, canvasW, canvasH, camW, camH, &m);
    int circ = p->imageType == 2 || p->imageType == 3;
    double centx = 0, centy = 0, sqrDist = 0;
    if (circ) {
        if (p->circleR > 0) {
            centx = p->circleX;
            centy = p->circleY;
            sqrDist = p->circleR * p->circleR;
        } else {
            centx = p->cropX + p->cropWidth / 2;
            centy = p->cropY + p->cropHeight / 2;
            sqrDist = p->cropWidth > p->cropHeight ? p->cropWidth * p->cropWidth * 0.25
                                                   : p->cropHeight * p->cropHeight * 0.25;
        }
    }
    for (int h = row0; h < row1; h++) {
        for (int w = 0; w < canvasW; w++) {
            double sx, sy;
            orc_remap_point(&m, w, h, &sx, &sy);
            int ok;
            if (!circ)
                ok = sx >= 0 && sy >= 0 && sx < camW && sy < camH;
            else
                ok = sx >= p->cropX && sy >= p->cropY && sx < p->cropX + p->cropWidth &&
                     sy < p->cropY + p->cropHeight &&
                     (sx - centx) * (sx - centx) + (sy - centy) * (sy - centy) < sqrDist;
            size_t idx = (size_t)h * canvasW + w;
            if (!ok) { sx = -1; sy = -1; }
            if (map64) { map64[2 * idx] = sx; map64[2 * idx + 1] = sy; }
            if (xmap) xmap[idx] = (float)sx;
            if (ymap) ymap[idx] = (float)sy;
            if (mask) mask[idx] = ok ? 255 : 0;
        }
    }
}

/* Nearest-optical-axis seam rule: a covered canvas pixel belongs to the
   covering camera whose optical axis makes the smallest angle with the
   pixel's ray; differences below 1e-12 rad count as ties and go to the lower
   camera index.  Keeps the invariants of getNonIntersectingMasks
   (source/Blend/Mask.cpp:376-398): seams_i is a subset of coverage_i and the
   seams partition the union of the coverages. */
void orc_nearest_axis_seams(const orc_param* params, int n, int camW, int camH, int canvasW, int canvasH,
                            const uint8_t* coverage, uint8_t* seams)
{
    orc_nearest_axis_seams_rows(params, n, camW, camH, canvasW, canvasH, 0, canvasH, coverage, seams);
}

void orc_nearest_axis_seams_rows(const orc_param* params, int n, int camW, int camH, int canvasW, int canvasH,
                                 int row0, int row1, const uint8_t* coverage, uint8_t* seams)
{
    size_t npx = (size_t)canvasW * canvasH;
    orc_remap* ms = (orc_remap*)malloc(sizeof(orc_remap) * (size_t)n);
    for (int i = 0; i < n; i++) orc_remap_init(&params[i], canvasW, canvasH, camW, camH, &ms[i]);
    for (int i = 0; i < n; i++)
        memset(seams + (size_t)i * npx + (size_t)row0 * canvasW, 0, (size_t)(row1 - row0) * canvasW);
    for (int h = row0; h < row1; h++) {
        for (int w = 0; w < canvasW; w++) {
            size_t idx = (size_t)h * canvasW + w;
            int best = -1;
            double bestAngle = 0;
            for (int i = 0; i < n; i++) {
                if (!coverage[(size_t)i * npx + idx]) continue;
                double a = orc_remap_axis_angle(&ms[i], w, h);
                if (best < 0 || a < bestAngle - 1e-12) { best = i; bestAngle = a; }
            }
            if (best >= 0) seams[(size_t)best * npx + idx] = 255;
        }
    }
    free(ms);
}

/* getLUT, source/Blend/ExposureColorOptimize.cpp:1217-1223:
   lut[v] = saturate_cast<uchar>(k * v), i.e. round half to even, clamp. */
void orc_get_lut(double k, uint8_t lut[256])
{
    for (int i = 0; i < 256; i++) {
        double v = nearbyint(k * i);
        lut[i] = v < 0 ? 0 : (v > 255 ? 255 : (uint8_t)v);
    }
}

/* ======================================================================== */
/* Remap: bilinearResampling + ZReprojectLoop, source/Warp/ZReproject.cpp    */
/* ======================================================================== */

/* saturate_cast<short>(double): cvRound (round half to even), clamp. */
static inline int16_t sat_round_short(double v)
{
    double r = nearbyint(v);
    if (r < -32768) return -32768;
    if (r > 32767) return 32767;
    return (int16_t)r;
}

/* One row range of the 16S reprojection.  The source pixels are the gain
   corrected ones (cudaTransform runs before the remap: source/Task/
   RicohUtil.cpp:1303-1309).  Bilinear weights and the sum order follow
   bilinearResampling (source/Warp/ZReproject.cpp:101-130); the right-hand
   tap column is clamped to W-1 (the reference reads x0+1 unclamped, past the
   row end, when x lies in [W-1, W)). */
void orc_reproject_bilinear_16s_rows(const uint8_t* src, int srcW, int srcH, long long srcStep, int channels,
                                     const uint8_t* lutted, const float* xmap, const float* ymap,
                                     int dstW, int row0, int row1, int16_t* dst)
{
    (void)lutted;
    for (int h = row0; h < row1; h++) {
        for (int w = 0; w < dstW; w++) {
            size_t idx = (size_t)h * dstW + w;
            double x = xmap[idx], y = ymap[idx];
            int16_t* o = dst + 4 * idx;
            o[0] = o[1] = o[2] = o[3] = 0;
            if (!(x >= 0 && y >= 0 && x < srcW && y < srcH)) continue;
            int x0 = (int)x, y0 = (int)y, x1 = x0 + 1, y1 = y0 + 1;
            if (x0 < 0) x0 = 0;
            if (x1 > srcW - 1) x1 = srcW - 1;
            if (y0 < 0) y0 = 0;
            if (y1 > srcH - 1) y1 = srcH - 1;
            double wx0 = x - x0, wx1 = 1 - wx0;
            double wy0 = y - y0, wy1 = 1 - wy0;
            double w00 = wx1 * wy1, w01 = wx0 * wy1;
            double w10 = wx1 * wy0, w11 = wx0 * wy0;
            const uint8_t* p00 = src + (size_t)y0 * srcStep + (size_t)x0 * channels;
            const uint8_t* p01 = src + (size_t)y0 * srcStep + (size_t)x1 * channels;
            const uint8_t* p10 = src + (size_t)y1 * srcStep + (size_t)x0 * channels;
            const uint8_t* p11 = src + (size_t)y1 * srcStep + (size_t)x1 * channels;
            for (int c = 0; c < 3; c++) {
                double res = 0;
                res += p00[c] * w00;
                res += p01[c] * w01;
                res += p10[c] * w10;
                res += p11[c] * w11;
                o[c] = sat_round_short(res);
            }
        }
    }
}

static void apply_lut(const uint8_t* src, int w, int h, long long step, int channels, const uint8_t* lut,
                      uint8_t* out /* tightly packed w*h*channels */)
{
    for (int y = 0; y < h; y++) {
        const uint8_t* s = src + (size_t)y * step;
        uint8_t* o = out + (size_t)y * w * channels;
        for (int x = 0; x < w; x++) {
            for (int c = 0; c < 3; c++) o[x * channels + c] = lut[c * 256 + s[x * channels + c]];
            if (channels == 4) o[x * channels + 3] = 0;
        }
    }
}

void orc_reproject_bilinear_16s(const uint8_t* src, int srcW, int srcH, long long srcStep, int channels,
                                const uint8_t* lut, const float* xmap, const float* ymap, int dstW, int dstH,
                                int16_t* dst)
{
    if (lut) {
        uint8_t* tmp = (uint8_t*)malloc((size_t)srcW * srcH * channels);
        apply_lut(src, srcW, srcH, srcStep, channels, lut, tmp);
        orc_reproject_bilinear_16s_rows(tmp, srcW, srcH, (long long)srcW * channels, channels, NULL, xmap, ymap,
                                        dstW, 0, dstH, dst);
        free(tmp);
    } else {
        orc_reproject_bilinear_16s_rows(src, srcW, srcH, srcStep, channels, NULL, xmap, ymap, dstW, 0, dstH, dst);
    }
}

/* ======================================================================== */
/* Pyramid primitives: source/CudaAccel/CudaPyramid2.cu, borders from        */
/* source/CudaAccel/CudaUtil.cuh:6-98 (vertical reflect-101, horizontal wrap) */
/* ======================================================================== */

/* BrdColReflect101::idx_row_low / idx_row_high (CudaUtil.cuh:28-48) */
static inline int row_low(int y, int H) { return abs(y) % H; }
static inline int row_high(int y, int H) { int last = H - 1; return abs(last - abs(last - y)) % H; }
/* BrdRowWrap::idx_col_low / idx_col_high (CudaUtil.cuh:50-74) */
static inline int col_low(int x, int W) { return x >= 0 ? x : x - ((x - W + 1) / W) * W; }
static inline int col_high(int x, int W) { return x < W ? x : x % W; }
static inline int col_any(int x, int W) { return col_high(col_low(x, W), W); }

static const int K5[5] = {1, 4, 6, 4, 1};

/* getTrueNumLevels, source/Blend/MultiBandBlend.cpp:329-337 */
int orc_num_levels(int width, int height, int maxLevels, int minLength)
{
    int numLevels = maxLevels < 0 ? 16 : (maxLevels > 16 ? 16 : maxLevels);
    int side = minLength < 0 ? 2 : (minLength > 64 ? 64 : minLength);
    int lw = (int)(log((double)width / side) / log(2.0));
    int lh = (int)(log((double)height / side) / log(2.0));
    int m = lw < lh ? lw : lh;
    return numLevels < m ? numLevels : m;
}

/* getPyramidLevelSizes, source/CudaAccel/CudaMultibandBlend.cpp:486-492 */
void orc_level_sizes(int w, int h, int levels, int* ws, int* hs)
{
    ws[0] = w;
    hs[0] = h;
    for (int i = 1; i <= levels; i++) {
        ws[i] = (ws[i - 1] + 1) / 2;
        hs[i] = (hs[i - 1] + 1) / 2;
    }
}

/* Row indices of the 5-tap decimation for output row y (pyrDown kernels,
   CudaPyramid2.cu:16-226: low mapping above, identity centre, high below). */
static inline void down_rows(int y, int H, int r[5])
{
    int sy = 2 * y;
    r[0] = row_low(sy - 2, H);
    r[1] = row_low(sy - 1, H);
    r[2] = sy;
    r[3] = row_high(sy + 1, H);
    r[4] = row_high(sy + 2, H);
}

/* Raw 5x5 sum S at output (x, y) of a C-channel int16 image (channels < nc
   are summed).  Row sums first, then columns, as the kernel does. */
static void down_sums_row(const int16_t* src, int sw, int sh, int C, int nc, int y, int dw, int32_t* out,
                          int32_t* vs /* (sw) * nc scratch */)
{
    int r[5];
    down_rows(y, sh, r);
    for (int x = 0; x < sw; x++)
        for (int c = 0; c < nc; c++) {
            int32_t s = 0;
            for (int k = 0; k < 5; k++) s += K5[k] * src[((size_t)r[k] * sw + x) * C + c];
            vs[x * nc + c] = s;
        }
    for (int x = 0; x < dw; x++)
        for (int c = 0; c < nc; c++) {
            int32_t s = 0;
            for (int k = 0; k < 5; k++) s += K5[k] * vs[col_any(2 * x + k - 2, sw) * nc + c];
            out[x * nc + c] = s;
        }
}

/* pyrDown16SC1To32SC1, CudaPyramid2.cu:16-122: raw sum */
void orc_pyr_down_16sc1_to_32sc1(const int16_t* src, int sw, int sh, int32_t* dst, int dw, int dh)
{
    int32_t* vs = (int32_t*)malloc(sizeof(int32_t) * (size_t)sw);
    for (int y = 0; y < dh; y++) down_sums_row(src, sw, sh, 1, 1, y, dw, dst + (size_t)y * dw, vs);
    free(vs);
}

/* pyrDown16SC1To16SC1, CudaPyramid2.cu:124-226: (S + 128) >> 8 */
void orc_pyr_down_16sc1_to_16sc1(const int16_t* src, int sw, int sh, int16_t* dst, int dw, int dh)
{
    int32_t* vs = (int32_t*)malloc(sizeof(int32_t) * (size_t)sw);
    int32_t* row = (int32_t*)malloc(sizeof(int32_t) * (size_t)dw);
    for (int y = 0; y < dh; y++) {
        down_sums_row(src, sw, sh, 1, 1, y, dw, row, vs);
        for (int x = 0; x < dw; x++) dst[(size_t)y * dw + x] = (int16_t)((row[x] + 128) >> 8);
    }
    free(row);
    free(vs);
}

/* pyrDown16SC4To16SC4 with scale, CudaPyramid2.cu:436-542:
   scale ? (S << 8) / scale : 0 per channel (C truncating division). */
void orc_pyr_down_16sc4_masked(const int16_t* src, int sw, int sh, const int32_t* scale, int16_t* dst, int dw,
                               int dh)
{
    int32_t* vs = (int32_t*)malloc(sizeof(int32_t) * (size_t)sw * 3);
    int32_t* row = (int32_t*)malloc(sizeof(int32_t) * (size_t)dw * 3);
    for (int y = 0; y < dh; y++) {
        down_sums_row(src, sw, sh, 4, 3, y, dw, row, vs);
        for (int x = 0; x < dw; x++) {
            int32_t s = scale[(size_t)y * dw + x];
            int16_t* o = dst + ((size_t)y * dw + x) * 4;
            for (int c = 0; c < 3; c++) o[c] = s ? (int16_t)((row[x * 3 + c] << 8) / s) : 0;
            o[3] = 0;
        }
    }
    free(row);
    free(vs);
}

/* Taps of the zero-inserted 2x upsample for output coordinate x (pyrUp
   kernels, CudaPyramid2.cu:544-710): even x -> (x/2-1, x/2, x/2+1) with
   weights (1, 6, 1); odd x -> ((x-1)/2, (x+1)/2) with weights (4, 4).
   Source indices outside [0, n) use the low / high border mapping. */
static inline int up_taps(int x, int* idx, int* wt)
{
    if ((x & 1) == 0) {
        idx[0] = x / 2 - 1; wt[0] = 1;
        idx[1] = x / 2;     wt[1] = 6;
        idx[2] = x / 2 + 1; wt[2] = 1;
        return 3;
    }
    idx[0] = (x - 1) / 2; wt[0] = 4;
    idx[1] = (x + 1) / 2; wt[1] = 4;
    return 2;
}

static inline int up_row(int r, int H) { return r < 0 ? row_low(r, H) : (r >= H ? row_high(r, H) : r); }
static inline int up_col(int c, int W) { return c < 0 ? col_low(c, W) : (c >= W ? col_high(c, W) : c); }

#define DEFINE_PYR_UP(NAME, T)                                                                          \
    void NAME(const T* src, int sw, int sh, T* dst, int dw, int dh)                                     \
    {                                                                                                   \
        int64_t* vs = (int64_t*)malloc(sizeof(int64_t) * (size_t)sw * 3);                               \
        for (int y = 0; y < dh; y++) {                                                                  \
            int ri[3], rw[3];                                                                           \
            int nr = up_taps(y, ri, rw);                                                                \
            for (int k = 0; k < nr; k++) ri[k] = up_row(ri[k], sh);                                     \
            for (int x = 0; x < sw; x++)                                                                \
                for (int c = 0; c < 3; c++) {                                                           \
                    int64_t s = 0;                                                                      \
                    for (int k = 0; k < nr; k++) s += (int64_t)rw[k] * src[((size_t)ri[k] * sw + x) * 4 + c]; \
                    vs[x * 3 + c] = s;                                                                  \
                }                                                                                       \
            for (int x = 0; x < dw; x++) {                                                              \
                int ci[3], cw[3];                                                                       \
                int nc = up_taps(x, ci, cw);                                                            \
                T* o = dst + ((size_t)y * dw + x) * 4;                                                  \
                for (int c = 0; c < 3; c++) {                                                           \
                    int32_t s = 0;                                                                      \
                    for (int k = 0; k < nc; k++) s += cw[k] * (int32_t)vs[up_col(ci[k], sw) * 3 + c];   \
                    o[c] = (T)((s + 32) >> 6);                                                          \
                }                                                                                       \
                o[3] = 0;                                                                               \
            }                                                                                           \
        }                                                                                               \
        free(vs);                                                                                       \
    }

DEFINE_PYR_UP(orc_pyr_up_16sc4, int16_t)
DEFINE_PYR_UP(orc_pyr_up_32sc4, int32_t)

/* ======================================================================== */
/* Multiband blend: CudaTilingMultibandBlendFast,                            */
/* source/CudaAccel/CudaMultibandBlend.cpp:549-642 (prepare), :785-823 (blend) */
/* ======================================================================== */

struct orc_blender {
    int n, W, H, L, full;
    int ws[17], hs[17];
    size_t off[18];        /* pixel offset of each level in a packed pyramid */
    int32_t* alpha;        /* n * total : alphaPyrs (level 0 unused) */
    int16_t* weight;       /* n * total : weightPyrs (or the custom masks' weights) */
    int32_t* wsum;         /* total : resultWeightPyr (only if !full) */
    uint8_t* masknot;      /* W*H (only if !full) */
    uint8_t* cov;          /* n*W*H : the prepared coverage masks */
    uint8_t* seams;        /* n*W*H : the prepared unique masks */
};

static size_t level_total(const orc_blender* b) { return b->off[b->L + 1]; }

/* Weight pyramids, weight sums and maskNot from the n weight masks `w`, with
   `uni_src` deciding maskNot (and fullMask): the prepared unique masks over
   the coverage (prepare, CudaMultibandBlend.cpp:586-642), or a set of custom
   masks (blend(images, masks, blendImage), :825-893: weights from the masks,
   the weighted normalisation whatever the coverage, maskNot from the masks'
   union). */
static void build_weights(orc_blender* b, const uint8_t* w, const uint8_t* uni_src, int custom)
{
    const int n = b->n;
    const size_t tot = level_total(b), npx = (size_t)b->W * b->H;
    for (int i = 0; i < n; i++) {
        int16_t* wt = b->weight + (size_t)i * tot;
        for (size_t p = 0; p < npx; p++) wt[p] = w[(size_t)i * npx + p] ? 256 : 0;
        for (int j = 0; j < b->L; j++)
            orc_pyr_down_16sc1_to_16sc1(wt + b->off[j], b->ws[j], b->hs[j], wt + b->off[j + 1], b->ws[j + 1],
                                        b->hs[j + 1]);
    }
    uint8_t* uni = (uint8_t*)calloc(npx, 1);
    size_t covered = 0;
    for (size_t p = 0; p < npx; p++) {
        for (int i = 0; i < n; i++)
            if (uni_src[(size_t)i * npx + p]) { uni[p] = 1; break; }
        covered += uni[p];
    }
    b->full = !custom && covered == npx;
    free(b->wsum);
    free(b->masknot);
    b->wsum = NULL;
    b->masknot = NULL;
    if (!b->full) {
        b->wsum = (int32_t*)calloc(tot, sizeof(int32_t));
        for (int i = 0; i < n; i++) {
            const int16_t* wt = b->weight + (size_t)i * tot;
            for (size_t p = 0; p < tot; p++) b->wsum[p] += wt[p];
        }
        b->masknot = (uint8_t*)malloc(npx);
        for (size_t p = 0; p < npx; p++) b->masknot[p] = uni[p] ? 0 : 255;
    }
    free(uni);
}

orc_blender* orc_mb_prepare(const uint8_t* masks, const uint8_t* seams, int n, int W, int H, int maxLevels,
                            int minLength)
{
    if (n <= 0 || n > 255 || W <= 0 || H <= 0) return NULL;
    orc_blender* b = (orc_blender*)calloc(1, sizeof(orc_blender));
    b->n = n;
    b->W = W;
    b->H = H;
    b->L = orc_num_levels(W, H, maxLevels, minLength);
    if (b->L < 0) b->L = 0;
    orc_level_sizes(W, H, b->L, b->ws, b->hs);
    b->off[0] = 0;
    for (int j = 0; j <= b->L; j++) b->off[j + 1] = b->off[j] + (size_t)b->ws[j] * b->hs[j];
    size_t tot = level_total(b), npx = (size_t)W * H;
    b->alpha = (int32_t*)calloc((size_t)n * tot, sizeof(int32_t));
    b->weight = (int16_t*)calloc((size_t)n * tot, sizeof(int16_t));
    b->cov = (uint8_t*)malloc((size_t)n * npx);
    b->seams = (uint8_t*)malloc((size_t)n * npx);
    memcpy(b->cov, masks, (size_t)n * npx);
    memcpy(b->seams, seams, (size_t)n * npx);
    int16_t* tmpAlpha = (int16_t*)malloc(sizeof(int16_t) * tot);
    for (int i = 0; i < n; i++) {
        int32_t* al = b->alpha + (size_t)i * tot;
        for (size_t p = 0; p < npx; p++) tmpAlpha[p] = masks[(size_t)i * npx + p] ? 256 : 0;
        for (int j = 0; j < b->L; j++) {
            orc_pyr_down_16sc1_to_32sc1(tmpAlpha + b->off[j], b->ws[j], b->hs[j], al + b->off[j + 1],
                                        b->ws[j + 1], b->hs[j + 1]);
            /* scaledSet16SC1Mask32SC1(temp, 256, alpha) */
            for (size_t p = b->off[j + 1]; p < b->off[j + 2]; p++) tmpAlpha[p] = al[p] ? 256 : 0;
        }
    }
    free(tmpAlpha);
    build_weights(b, seams, masks, 0);
    return b;
}

int orc_mb_set_custom_masks(orc_blender* b, const uint8_t* masks)
{
    if (masks) build_weights(b, masks, masks, 1);
    else build_weights(b, b->seams, b->cov, 0);
    return 0;
}

void orc_mb_free(orc_blender* b)
{
    if (!b) return;
    free(b->alpha);
    free(b->weight);
    free(b->wsum);
    free(b->masknot);
    free(b->cov);
    free(b->seams);
    free(b);
}

int orc_mb_num_levels(const orc_blender* b) { return b->L; }
int orc_mb_full_mask(const orc_blender* b) { return b->full; }

void orc_mb_get_alpha(const orc_blender* b, int cam, int level, int32_t* out)
{
    size_t tot = level_total(b);
    memcpy(out, b->alpha + (size_t)cam * tot + b->off[level], sizeof(int32_t) * (b->off[level + 1] - b->off[level]));
}

void orc_mb_get_weight(const orc_blender* b, int cam, int level, int16_t* out)
{
    size_t tot = level_total(b);
    memcpy(out, b->weight + (size_t)cam * tot + b->off[level], sizeof(int16_t) * (b->off[level + 1] - b->off[level]));
}

/* Laplacian pyramid of camera i (tile(), CudaMultibandBlend.cpp:762-783):
   G_{j+1} = masked pyrDown(G_j, alpha_{j+1}); L_j = G_j - pyrUp(G_{j+1});
   L_L = G_L.  lap holds 4 int16 per pixel, levels packed by off[]. */
static void build_laplacian(const orc_blender* b, int i, const int16_t* image, int16_t* lap, int16_t* up)
{
    size_t tot = level_total(b);
    const int32_t* al = b->alpha + (size_t)i * tot;
    memcpy(lap, image, sizeof(int16_t) * 4 * (size_t)b->W * b->H);
    for (int j = 0; j < b->L; j++)
        orc_pyr_down_16sc4_masked(lap + 4 * b->off[j], b->ws[j], b->hs[j], al + b->off[j + 1],
                                  lap + 4 * b->off[j + 1], b->ws[j + 1], b->hs[j + 1]);
    for (int j = 0; j < b->L; j++) {
        orc_pyr_up_16sc4(lap + 4 * b->off[j + 1], b->ws[j + 1], b->hs[j + 1], up, b->ws[j], b->hs[j]);
        int16_t* g = lap + 4 * b->off[j];
        size_t np = (size_t)b->ws[j] * b->hs[j];
        for (size_t p = 0; p < np; p++) {
            for (int c = 0; c < 3; c++) g[4 * p + c] = (int16_t)(g[4 * p + c] - up[4 * p + c]);
            g[4 * p + 3] = 0;
        }
    }
}

/* accumulate16SC4To32SC4 (CudaPyramid2.cu:736-747) over pixel range [p0,p1) */
static void accumulate_range(const orc_blender* b, int i, const int16_t* lap, int32_t* res, size_t p0, size_t p1)
{
    const int16_t* wt = b->weight + (size_t)i * level_total(b);
    for (size_t p = p0; p < p1; p++) {
        int w = wt[p];
        for (int c = 0; c < 3; c++) res[4 * p + c] += w * lap[4 * p + c];
    }
}

/* normalize32SC4, CudaPyramid2.cu:749-757 (full mask) and :775-791 */
static void normalize_range(const orc_blender* b, int32_t* res, size_t p0, size_t p1)
{
    for (size_t p = p0; p < p1; p++) {
        int32_t* r = res + 4 * p;
        if (b->full) {
            for (int c = 0; c < 3; c++) r[c] = (r[c] + 128) >> 8;
        } else {
            int w = b->wsum[p];
            if (!w) w++;
            for (int c = 0; c < 3; c++) r[c] /= w;
        }
        r[3] = 0;
    }
}

/* restoreImageFromLaplacePyramid (CudaMultibandBlend.cpp:220-231) and the
   8-bit conversion + maskNot zeroing (:820-822). */
static void collapse_and_output(const orc_blender* b, int32_t* res, uint8_t* dst, int32_t* coll_out)
{
    int32_t* up = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)b->W * b->H);
    for (int j = b->L; j > 0; j--) {
        orc_pyr_up_32sc4(res + 4 * b->off[j], b->ws[j], b->hs[j], up, b->ws[j - 1], b->hs[j - 1]);
        int32_t* r = res + 4 * b->off[j - 1];
        size_t np = (size_t)b->ws[j - 1] * b->hs[j - 1];
        for (size_t p = 0; p < np; p++)
            for (int c = 0; c < 3; c++) r[4 * p + c] += up[4 * p + c];
    }
    free(up);
    if (coll_out) memcpy(coll_out, res, sizeof(int32_t) * 4 * level_total(b));
    size_t npx = (size_t)b->W * b->H;
    for (size_t p = 0; p < npx; p++) {
        uint8_t* o = dst + 4 * p;
        if (!b->full && b->masknot[p]) {
            o[0] = o[1] = o[2] = o[3] = 0;
            continue;
        }
        for (int c = 0; c < 3; c++) {
            int32_t v = res[4 * p + c];
            o[c] = v < 0 ? 0 : (v > 255 ? 255 : (uint8_t)v);
        }
        o[3] = 0;
    }
}

void orc_mb_blend(orc_blender* b, const int16_t* const* images, uint8_t* dst, int32_t* norm_out, int32_t* coll_out)
{
    size_t tot = level_total(b);
    int32_t* res = (int32_t*)calloc(4 * tot, sizeof(int32_t));
    int16_t* lap = (int16_t*)malloc(sizeof(int16_t) * 4 * tot);
    int16_t* up = (int16_t*)malloc(sizeof(int16_t) * 4 * (size_t)b->W * b->H);
    for (int i = 0; i < b->n; i++) {
        build_laplacian(b, i, images[i], lap, up);
        accumulate_range(b, i, lap, res, 0, tot);
    }
    normalize_range(b, res, 0, tot);
    if (norm_out) memcpy(norm_out, res, sizeof(int32_t) * 4 * tot);
    collapse_and_output(b, res, dst, coll_out);
    free(up);
    free(lap);
    free(res);
}

/* ---- multithreaded variant: camera-parallel pyramids (like
   TilingMultibandBlendFastParallel, source/Blend/MultiBandBlend.cpp:
   1430-1482), then row-parallel accumulation.  Integer sums make the result
   identical to orc_mb_blend. */
typedef struct {
    orc_blender* b;
    const int16_t* const* images;
    int16_t* laps;
    int32_t* res;
    int tid, nthreads;
} mt_ctx;

static void* mt_lap_worker(void* arg)
{
    mt_ctx* c = (mt_ctx*)arg;
    size_t tot = level_total(c->b);
    int16_t* up = (int16_t*)malloc(sizeof(int16_t) * 4 * (size_t)c->b->W * c->b->H);
    for (int i = c->tid; i < c->b->n; i += c->nthreads)
        build_laplacian(c->b, i, c->images[i], c->laps + (size_t)i * 4 * tot, up);
    free(up);
    return NULL;
}

static void* mt_acc_worker(void* arg)
{
    mt_ctx* c = (mt_ctx*)arg;
    size_t tot = level_total(c->b);
    size_t chunk = (tot + c->nthreads - 1) / c->nthreads;
    size_t p0 = chunk * c->tid, p1 = p0 + chunk > tot ? tot : p0 + chunk;
    if (p0 >= p1) return NULL;
    for (int i = 0; i < c->b->n; i++) accumulate_range(c->b, i, c->laps + (size_t)i * 4 * tot, c->res, p0, p1);
    normalize_range(c->b, c->res, p0, p1);
    return NULL;
}

static void run_threads(void* (*fn)(void*), mt_ctx* ctx, int nthreads)
{
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, fn, &ctx[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
}

void orc_mb_blend_mt(orc_blender* b, const int16_t* const* images, uint8_t* dst, int nthreads)
{
    if (nthreads <= 1) { orc_mb_blend(b, images, dst, NULL, NULL); return; }
    size_t tot = level_total(b);
    int16_t* laps = (int16_t*)malloc(sizeof(int16_t) * 4 * tot * (size_t)b->n);
    int32_t* res = (int32_t*)calloc(4 * tot, sizeof(int32_t));
    mt_ctx* ctx = (mt_ctx*)malloc(sizeof(mt_ctx) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        ctx[t].b = b; ctx[t].images = images; ctx[t].laps = laps; ctx[t].res = res;
        ctx[t].tid = t; ctx[t].nthreads = nthreads;
    }
    run_threads(mt_lap_worker, ctx, nthreads);
    run_threads(mt_acc_worker, ctx, nthreads);
    collapse_and_output(b, res, dst, NULL);
    free(ctx);
    free(res);
    free(laps);
}

/* ---- whole render ------------------------------------------------------ */
typedef struct {
    const uint8_t* src;
    int srcW, srcH, channels;
    const float *xmap, *ymap;
    int dstW, row0, row1;
    int16_t* dst;
} remap_job;

static void* remap_worker(void* arg)
{
    remap_job* j = (remap_job*)arg;
    orc_reproject_bilinear_16s_rows(j->src, j->srcW, j->srcH, (long long)j->srcW * j->channels, j->channels, NULL,
                                    j->xmap, j->ymap, j->dstW, j->row0, j->row1, j->dst);
    return NULL;
}

void orc_render(orc_blender* b, const uint8_t* const* srcs, int srcW, int srcH, int channels, const uint8_t* luts,
                const float* const* xmaps, const float* const* ymaps, uint8_t* dst, int nthreads)
{
    int n = b->n;
    if (nthreads < 1) nthreads = 1;
    size_t npx = (size_t)b->W * b->H;
    int16_t** imgs = (int16_t**)calloc((size_t)n, sizeof(int16_t*));
    uint8_t* tmp = (uint8_t*)malloc((size_t)srcW * srcH * channels);
    remap_job* jobs = (remap_job*)malloc(sizeof(remap_job) * (size_t)nthreads);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int i = 0; i < n; i++) {
        imgs[i] = (int16_t*)malloc(sizeof(int16_t) * 4 * npx);
        const uint8_t* s = srcs[i];
        if (luts) {
            apply_lut(srcs[i], srcW, srcH, (long long)srcW * channels, channels, luts + (size_t)i * 768, tmp);
            s = tmp;
        }
        int rows = (b->H + nthreads - 1) / nthreads;
        for (int t = 0; t < nthreads; t++) {
            remap_job* j = &jobs[t];
            j->src = s; j->srcW = srcW; j->srcH = srcH; j->channels = channels;
            j->xmap = xmaps[i]; j->ymap = ymaps[i]; j->dstW = b->W;
            j->row0 = t * rows < b->H ? t * rows : b->H;
            j->row1 = (t + 1) * rows < b->H ? (t + 1) * rows : b->H;
            j->dst = imgs[i];
        }
        if (nthreads == 1) remap_worker(&jobs[0]);
        else {
            for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, remap_worker, &jobs[t]);
            for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
        }
    }
    orc_mb_blend_mt(b, (const int16_t* const*)imgs, dst, nthreads);
    for (int i = 0; i < n; i++) free(imgs[i]);
    free(th);
    free(jobs);
    free(tmp);
    free(imgs);
}

/* ---- encoder handoff: BGR32 -> YUV420P / NV12 ------------------------------
 * source/CudaAccel/ImageProc.cu:44-95 (cvtBGRToYUV2x2Block) over 2x2 blocks
 * (:97-117).  BT.601 coefficients scaled by 2^20, +0.5 rounding and the
 * 16 / 128 offsets folded in; every sum is non-negative, so >> is a floor.
 * Luma per pixel; chroma of a block from its left column only (top-left and
 * bottom-left pixels), averaged by one extra shift.
 */
static int yuv_clamp(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }

static int yuv_y(const uint8_t* p)
{
    return yuv_clamp((269484 * p[2] + 528482 * p[1] + 102760 * p[0] + (1 << 19) + (16 << 20)) >> 20);
}

static void yuv_uv_sums(const uint8_t* p, int* su, int* sv)
{
    *su = -155188 * p[2] - 305135 * p[1] + 460324 * p[0] + (1 << 19) + (128 << 20);
    *sv = 460324 * p[2] - 385875 * p[1] - 74448 * p[0] + (1 << 19) + (128 << 20);
}

void orc_bgr32_to_yuv(const uint8_t* bgr, long long bgrStep, int w, int h, int fmt, uint8_t* y, long long yStep,
                      uint8_t* u, long long uStep, uint8_t* v, long long vStep)
{
    for (int by = 0; by < h / 2; by++) {
        const uint8_t* top = bgr + (size_t)(2 * by) * bgrStep;
        const uint8_t* bot = top + bgrStep;
        uint8_t* yt = y + (size_t)(2 * by) * yStep;
        uint8_t* yb = yt + yStep;
        for (int bx = 0; bx < w / 2; bx++) {
            const int x = 2 * bx;
            yt[x] = (uint8_t)yuv_y(top + 4 * x);
            yt[x + 1] = (uint8_t)yuv_y(top + 4 * x + 4);
            yb[x] = (uint8_t)yuv_y(bot + 4 * x);
            yb[x + 1] = (uint8_t)yuv_y(bot + 4 * x + 4);
            int u0, v0, u1, v1;
            yuv_uv_sums(top + 4 * x, &u0, &v0);
            yuv_uv_sums(bot + 4 * x, &u1, &v1);
            const uint8_t cu = (uint8_t)yuv_clamp((u0 + u1) >> 21), cv = (uint8_t)yuv_clamp((v0 + v1) >> 21);
            if (fmt == 12) {
                u[(size_t)by * uStep + x] = cu;
                u[(size_t)by * uStep + x + 1] = cv;
            } else {
                u[(size_t)by * uStep + bx] = cu;
                v[(size_t)by * vStep + bx] = cv;
            }
        }
    }
}

/* ---- decoder frames: YUV420P / NV12 -> BGR32 ------------------------------
 * source/CudaAccel/ImageProc.cu:165-222 (cvtYUV2x2BlockToBGR over 2x2
 * blocks): u = U - 128, v = V - 128, y' = max(Y - 16, 0) * 1220542; each
 * channel is (y' + 2^19 + chroma term) >> 20 clamped to 0..255, with the
 * chroma terms 1673527 v (R), -852492 v - 409993 u (G), 2116026 u (B).  The
 * device's >> of a negative int is a floor; floor_shift20 states it without
 * relying on C's implementation-defined shift of negative values.  The
 * fourth byte is written 0.
 */
static int floor_shift20(int v) { return v >= 0 ? v >> 20 : -((-v + (1 << 20) - 1) >> 20); }

static void yuv_to_bgr_px(int yv, int ruv, int guv, int buv, uint8_t* o)
{
    const int yy = (yv > 16 ? yv - 16 : 0) * 1220542;
    o[0] = (uint8_t)yuv_clamp(floor_shift20(yy + buv));
    o[1] = (uint8_t)yuv_clamp(floor_shift20(yy + guv));
    o[2] = (uint8_t)yuv_clamp(floor_shift20(yy + ruv));
    o[3] = 0;
}

void orc_yuv_to_bgr32(const uint8_t* y, long long yStep, const uint8_t* u, long long uStep, const uint8_t* v,
                      long long vStep, int w, int h, int fmt, uint8_t* bgr, long long bgrStep)
{
    for (int by = 0; by < h / 2; by++)
        for (int bx = 0; bx < w / 2; bx++) {
            const int x = 2 * bx, yr = 2 * by;
            int cu, cv;
            if (fmt == 12) {
                cu = u[(size_t)by * uStep + x];
                cv = u[(size_t)by * uStep + x + 1];
            } else {
                cu = u[(size_t)by * uStep + bx];
                cv = v[(size_t)by * vStep + bx];
            }
            cu -= 128;
            cv -= 128;
            const int ruv = (1 << 19) + 1673527 * cv;
            const int guv = (1 << 19) - 852492 * cv - 409993 * cu;
            const int buv = (1 << 19) + 2116026 * cu;
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 2; c++)
                    yuv_to_bgr_px(y[(size_t)(yr + r) * yStep + x + c], ruv, guv, buv,
                                  bgr + (size_t)(yr + r) * bgrStep + 4 * (size_t)(x + c));
        }
}

/* ---- getNonIntersectingMasks (source/Blend/Mask.cpp:376-398) ---------------
 * Distance transform: OpenCV 3.0's cv::distanceTransform with CV_DIST_L1 and
 * a 3x3 mask is a two-pass chamfer (forward: up-left, up, up-right, left;
 * backward: down-right, down, down-left, right) with step 1 for horizontal /
 * vertical and 2 for diagonal neighbours, which yields the exact L1 distance
 * to the nearest zero pixel.  Outside the image counts as far away.
 */
void orc_distance_transform_l1(const uint8_t* mask, int W, int H, int32_t* d)
{
    const int32_t far = ORC_DT_FAR;
#define DT_AT(y, x) (((y) < 0 || (y) >= H || (x) < 0 || (x) >= W) ? far : d[(size_t)(y) * W + (x)])
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            size_t o = (size_t)y * W + x;
            if (!mask[o]) {
                d[o] = 0;
                continue;
            }
            int32_t v = DT_AT(y - 1, x - 1) + 2, t;
            if ((t = DT_AT(y - 1, x) + 1) < v) v = t;
            if ((t = DT_AT(y - 1, x + 1) + 2) < v) v = t;
            if ((t = DT_AT(y, x - 1) + 1) < v) v = t;
            d[o] = v;
        }
    for (int y = H - 1; y >= 0; y--)
        for (int x = W - 1; x >= 0; x--) {
            size_t o = (size_t)y * W + x;
            int32_t v = d[o], t;
            if (v <= 1) continue;
            if ((t = DT_AT(y + 1, x + 1) + 2) < v) v = t;
            if ((t = DT_AT(y + 1, x) + 1) < v) v = t;
            if ((t = DT_AT(y + 1, x - 1) + 2) < v) v = t;
            if ((t = DT_AT(y, x + 1) + 1) < v) v = t;
            d[o] = v;
        }
#undef DT_AT
}

void orc_non_intersecting_masks(const uint8_t* masks, int n, int W, int H, uint8_t* out)
{
    const size_t npx = (size_t)W * H;
    uint8_t* uni = (uint8_t*)malloc(npx);
    int32_t* dist = (int32_t*)malloc(npx * sizeof(int32_t));
    int32_t* cur = (int32_t*)malloc(npx * sizeof(int32_t));
    for (int i = 0; i < n; i++)
        for (size_t p = 0; p < npx; p++) out[i * npx + p] = masks[i * npx + p] ? 255 : 0;
    memcpy(uni, out, npx);
    for (int i = 1; i < n; i++) {
        orc_distance_transform_l1(uni, W, H, dist);
        orc_distance_transform_l1(out + i * npx, W, H, cur);
        for (size_t p = 0; p < npx; p++) {
            const uint8_t take = cur[p] > dist[p] ? 255 : 0;
            out[i * npx + p] = take;
            if (take) {
                for (int j = 0; j < i; j++) out[j * npx + p] = 0;
                uni[p] = 255;
            }
        }
    }
    free(uni);
    free(dist);
    free(cur);
}

/* ---- linear blend --------------------------------------------------------
 * Weights: getWeightsLinearBlend32F (source/Blend/LinearBlend.cpp:136-151).
 * cv::GaussianBlur(unique, dist, Size(2r+1, 2r+1), r/3., r/3.) on an 8-bit
 * mask: cv::getGaussianKernel's terms exp(-x^2 / (2 sigma^2)) are stored as
 * float, normalised by their (double) sum into float, scaled by 2^8 and
 * rounded to integers; rows then columns are filtered with the integer taps
 * (border reflect-101, repeated for radii beyond the image), and the
 * 2^16-scaled sum is rounded and saturated to 8 bits.  cv::bitwise_and with
 * the 0/255 coverage keeps the blurred value where covered.  calcWeights32F
 * (:78-120): where two or more cameras are non-zero, w_k = d_k * (1 / sum),
 * one fp32 reciprocal and one product; where exactly one is, 1.
 */
static void linear_taps(int r, int* q)
{
    const int n = 2 * r + 1;
    const double sigma = r / 3.0, scale2X = -0.5 / (sigma * sigma);
    float* f = (float*)malloc(sizeof(float) * (size_t)n);
    double sum = 0;
    for (int i = 0; i < n; i++) {
        const double x = i - (n - 1) * 0.5;
        f[i] = (float)exp(scale2X * x * x);
        sum += f[i];
    }
    sum = 1. / sum;
    for (int i = 0; i < n; i++) {
        const float k = (float)(f[i] * sum);
        q[i] = (int)nearbyint((double)k * 256.0);
    }
    free(f);
}

static int reflect101_index(int p, int len)
{
    if (len == 1) return 0;
    while (p < 0 || p >= len) p = p < 0 ? -p : 2 * len - 2 - p;
    return p;
}

void orc_linear_weights(const uint8_t* cov, const uint8_t* seams, int n, int W, int H, int r, float* w)
{
    const size_t npx = (size_t)W * H;
    int* q = (int*)malloc(sizeof(int) * (size_t)(2 * r + 1));
    linear_taps(r, q);
    int32_t* rows = (int32_t*)malloc(sizeof(int32_t) * npx);
    uint8_t* dist = (uint8_t*)malloc(npx * (size_t)n);
    for (int c = 0; c < n; c++) {
        const uint8_t* s = seams + (size_t)c * npx;
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                int acc = 0;
                for (int k = 0; k <= 2 * r; k++) acc += q[k] * (s[(size_t)y * W + reflect101_index(x + k - r, W)] ? 255 : 0);
                rows[(size_t)y * W + x] = acc;
            }
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                long long acc = 0;
                for (int k = 0; k <= 2 * r; k++) acc += (long long)q[k] * rows[(size_t)reflect101_index(y + k - r, H) * W + x];
                long long v = (acc + (1 << 15)) >> 16;
                if (v < 0) v = 0;
                if (v > 255) v = 255;
                const size_t o = (size_t)c * npx + (size_t)y * W + x;
                dist[o] = (uint8_t)v & (cov[o] ? 255 : 0);
            }
    }
    for (size_t p = 0; p < npx; p++) {
        float sum = 0.f;
        int count = 0, last = 0;
        for (int k = 0; k < n; k++) {
            const int d = dist[(size_t)k * npx + p];
            sum += (float)d;
            if (d) {
                count++;
                last = k;
            }
        }
        const float inv = count > 1 ? 1.0f / sum : 0.f;
        for (int k = 0; k < n; k++) {
            float v = 0.f;
            if (count > 1) v = (float)dist[(size_t)k * npx + p] * inv;
            else if (count == 1 && k == last) v = 1.f;
            w[(size_t)k * npx + p] = v;
        }
    }
    free(q);
    free(rows);
    free(dist);
}

void orc_linear_render(const uint8_t* const* srcs, int srcW, int srcH, int channels, const uint8_t* luts,
                       const float* const* xmaps, const float* const* ymaps, const float* weights, int n, int W,
                       int H, uint8_t* dst)
{
    const size_t npx = (size_t)W * H;
    float* acc = (float*)calloc(npx * 3, sizeof(float));
    int16_t* img = (int16_t*)malloc(sizeof(int16_t) * 4 * npx);
    for (int i = 0; i < n; i++) {
        orc_reproject_bilinear_16s(srcs[i], srcW, srcH, (long long)srcW * channels, channels,
                                   luts ? luts + (size_t)i * 768 : NULL, xmaps[i], ymaps[i], W, H, img);
        const float* wi = weights + (size_t)i * npx;
        for (size_t p = 0; p < npx; p++) {
            /* reprojectWeightedAccumulateTo32F adds only where the map is valid */
            const float x = xmaps[i][p], y = ymaps[i][p];
            if (!(x >= 0 && y >= 0 && x < srcW && y < srcH)) continue;
            for (int c = 0; c < 3; c++) {
                const float prod = (float)img[4 * p + c] * wi[p];
                acc[3 * p + c] = acc[3 * p + c] + prod;
            }
        }
    }
    for (size_t p = 0; p < npx; p++) {
        for (int c = 0; c < 3; c++) {
            const float v = nearbyintf(acc[3 * p + c]);
            dst[4 * p + c] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
        }
        dst[4 * p + 3] = 0;
    }
    free(acc);
    free(img);
}
