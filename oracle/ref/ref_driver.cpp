/*
 * ref_driver.cpp -- C entry points over the reference's own code, for
 * pinning the oracle (oracle/ps_oracle.c) against it.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile's `ref` target compiles, from
 * the reference tree where it lies, these unchanged sources into
 * oracle/_ref/libpsref.so together with this file:
 *   - source/Warp/Remap.cpp and source/Warp/ZReproject.cpp (geometry, maps,
 *     the CPU bilinear remap), against the OpenCV subset in cv_shim/;
 *   - source/CudaAccel/CudaPyramid2.cu (every integer pyramid kernel and its
 *     host wrapper) and source/CudaAccel/ImageProc.cu (the YUV conversions),
 *     run on host cores by cuda_emu/.
 * Only the orchestration below is written here: it calls the reference's
 * functions in the order the reference's own callers do, citing them.
 */
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "ZReproject.h"
#include "opencv2/core.hpp"
#include "opencv2/core/cuda.hpp"

/* The reference's pyramid wrappers (declared in
   source/CudaAccel/CudaPyramid.h:6-33, defined in CudaPyramid2.cu). */
void pyramidDown16SC1To16SC1(const cv::cuda::GpuMat& src, cv::cuda::GpuMat& dst, cv::Size dstSize, bool horiWrap,
                             cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void pyramidDown16SC1To32SC1(const cv::cuda::GpuMat& src, cv::cuda::GpuMat& dst, cv::Size dstSize, bool horiWrap,
                             cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void pyramidDown16SC4To16SC4(const cv::cuda::GpuMat& src, const cv::cuda::GpuMat& scale, cv::cuda::GpuMat& dst,
                             bool horiWrap, cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void pyramidUp16SC4To16SC4(const cv::cuda::GpuMat& src, cv::cuda::GpuMat& dst, cv::Size dstSize, bool horiWrap,
                           cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void pyramidUp32SC4To32SC4(const cv::cuda::GpuMat& src, cv::cuda::GpuMat& dst, cv::Size dstSize, bool horiWrap,
                           cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void accumulate16SC4To32SC4(const cv::cuda::GpuMat& src, const cv::cuda::GpuMat& weight, cv::cuda::GpuMat& dst,
                            cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void normalize32SC4(cv::cuda::GpuMat& image, cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void normalize32SC4(cv::cuda::GpuMat& image, const cv::cuda::GpuMat& weight,
                    cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void scaledSet16SC1Mask32SC1(cv::cuda::GpuMat& image, short val, const cv::cuda::GpuMat& mask,
                             cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void subtract16SC4(const cv::cuda::GpuMat& a, const cv::cuda::GpuMat& b, cv::cuda::GpuMat& c,
                   cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void add32SC4(const cv::cuda::GpuMat& a, const cv::cuda::GpuMat& b, cv::cuda::GpuMat& c,
              cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void accumulate16SC1To32SC1(const cv::cuda::GpuMat& src, cv::cuda::GpuMat& dst,
                            cv::cuda::Stream& stream = cv::cuda::Stream::Null());

/* The reference's colour conversions (declared in
   source/CudaAccel/CudaInterface.h:161-171, defined in ImageProc.cu). */
void cvtBGR32ToYUV420P(const cv::cuda::GpuMat& bgr32, cv::cuda::GpuMat& y, cv::cuda::GpuMat& u,
                       cv::cuda::GpuMat& v, cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void cvtBGR32ToNV12(const cv::cuda::GpuMat& bgr32, cv::cuda::GpuMat& y, cv::cuda::GpuMat& uv,
                    cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void cvtYUV420PToBGR32(const cv::cuda::GpuMat& y, const cv::cuda::GpuMat& u, const cv::cuda::GpuMat& v,
                       cv::cuda::GpuMat& bgr32, cv::cuda::Stream& stream = cv::cuda::Stream::Null());
void cvtNV12ToBGR32(const cv::cuda::GpuMat& y, const cv::cuda::GpuMat& uv, cv::cuda::GpuMat& bgr32,
                    cv::cuda::Stream& stream = cv::cuda::Stream::Null());

/* PhotoParam's constructor lives in source/Warp/PhotoParam.cpp:9-12, a file
   that needs ticpp; it zeroes every field. */
PhotoParam::PhotoParam() { std::memset(this, 0, sizeof(PhotoParam)); }

namespace cv {
void parallel_for_(const Range& range, const ParallelLoopBody& body, double)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int r = range.start; r < range.end; ++r) body(Range(r, r + 1));
}
}  // namespace cv

namespace {

/* Same field order as PhotoParam (source/Warp/ZReproject.h:17-50). */
struct RefParam {
    int imageType, cropMode, cropX, cropY, cropWidth, cropHeight;
    int circleX, circleY, circleR;
    double hfov, vfov, alpha, beta, gamma, shiftX, shiftY, shearX, shearY;
    double yaw, pitch, roll;
};

PhotoParam toPhotoParam(const RefParam& r)
{
    PhotoParam p;
    p.imageType = r.imageType;
    p.cropMode = r.cropMode;
    p.cropX = r.cropX;
    p.cropY = r.cropY;
    p.cropWidth = r.cropWidth;
    p.cropHeight = r.cropHeight;
    p.circleX = r.circleX;
    p.circleY = r.circleY;
    p.circleR = r.circleR;
    p.hfov = r.hfov;
    p.vfov = r.vfov;
    p.alpha = r.alpha;
    p.beta = r.beta;
    p.gamma = r.gamma;
    p.shiftX = r.shiftX;
    p.shiftY = r.shiftY;
    p.shearX = r.shearX;
    p.shearY = r.shearY;
    p.yaw = r.yaw;
    p.pitch = r.pitch;
    p.roll = r.roll;
    return p;
}

template <class T>
void copyOut(const cv::Mat& m, T* out)
{
    const size_t row = (size_t)m.cols * m.elemSize();
    for (int r = 0; r < m.rows; ++r) std::memcpy((uint8_t*)out + row * r, m.ptr(r), row);
}

cv::Mat copyIn(const void* data, int rows, int cols, int type)
{
    cv::Mat m(rows, cols, type);
    const size_t row = (size_t)cols * m.elemSize();
    for (int r = 0; r < rows; ++r) std::memcpy(m.ptr(r), (const uint8_t*)data + row * r, row);
    return m;
}

size_t levelPixels(int W, int H, int levels)
{
    size_t n = 0;
    for (int j = 0; j <= levels; ++j) {
        n += (size_t)W * H;
        W = (W + 1) / 2;
        H = (H + 1) / 2;
    }
    return n;
}

}  // namespace

extern "C" {

int psref_num_threads(int n)
{
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

/* getReprojectMapAndMask (source/Warp/ZReproject.cpp:132-219): the CV_64FC2
   dst->src map (-1 where not covered) and the 0/255 coverage mask. */
int psref_reproject_map(const RefParam* param, int srcW, int srcH, int dstW, int dstH, double* map, uint8_t* mask)
{
    try {
        cv::Mat m, k;
        getReprojectMapAndMask(toPhotoParam(*param), cv::Size(srcW, srcH), cv::Size(dstW, dstH), m, k);
        copyOut(m, map);
        copyOut(k, mask);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

/* reprojectParallelTo16S (source/Warp/ZReproject.cpp:535-567): bilinear
   samples of an 8-bit image with `channels` channels through a CV_64FC2
   map into int16 (0 where the map is outside the source). */
int psref_reproject_16s(const uint8_t* src, int srcW, int srcH, int channels, const double* map, int dstW, int dstH,
                        int16_t* dst)
{
    try {
        cv::Mat s = copyIn(src, srcH, srcW, CV_MAKETYPE(CV_8U, channels));
        cv::Mat m = copyIn(map, dstH, dstW, CV_64FC2);
        cv::Mat d;
        reprojectParallelTo16S(s, d, m);
        copyOut(d, dst);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

/* CudaTilingMultibandBlendFast::prepare (source/CudaAccel/CudaMultibandBlend.cpp:549-642)
   followed by ::blend (:785-823), with the reference's pyramid wrappers.
   Inputs: n coverage masks and n unique (seam) masks, each W*H bytes
   (0 / non-zero), and n level-0 images of W*H int16x4.  `levels` is the
   numLevels that getTrueNumLevels would return.  The unique masks are
   given instead of computed by getNonIntersectingMasks (:570-571).
   Outputs (nullable except blend): blend W*H*4 bytes; coll / norm the
   collapsed and the normalised int32x4 result pyramids, levels 0..L packed;
   weights n int16 weight pyramids; alphas n int32 alpha pyramids (level 0
   left zero, as the reference keeps no level-0 alpha). */
int psref_mb_blend(int n, int W, int H, int levels, const uint8_t* masks, const uint8_t* uniq,
                   const int16_t* images, uint8_t* blend, int32_t* coll, int32_t* norm, int16_t* weights,
                   int32_t* alphas)
{
    try {
        const int rows = H, cols = W, numImages = n, numLevels = levels;
        const size_t px = (size_t)W * H;
        std::vector<cv::cuda::GpuMat> uniqueMasks(numImages), masksGpu(numImages);
        for (int i = 0; i < numImages; i++) {
            uniqueMasks[i].upload(copyIn(uniq + px * i, rows, cols, CV_8UC1));
            masksGpu[i].upload(copyIn(masks + px * i, rows, cols, CV_8UC1));
        }

        /* prepare: :580-604 */
        cv::cuda::GpuMat aux16S(rows, cols, CV_16SC1);
        std::vector<cv::cuda::GpuMat> tempAlphaPyr(numLevels + 1);
        std::vector<std::vector<cv::cuda::GpuMat>> alphaPyrs(numImages), weightPyrs(numImages);
        for (int i = 0; i < numImages; i++) {
            alphaPyrs[i].resize(numLevels + 1);
            weightPyrs[i].resize(numLevels + 1);
            aux16S.setTo(0);
            aux16S.setTo(256, masksGpu[i]);
            tempAlphaPyr[0] = aux16S.clone();
            aux16S.setTo(0);
            aux16S.setTo(256, uniqueMasks[i]);
            weightPyrs[i][0] = aux16S.clone();
            for (int j = 0; j < numLevels; j++) {
                pyramidDown16SC1To32SC1(tempAlphaPyr[j], alphaPyrs[i][j + 1], cv::Size(), true);
                tempAlphaPyr[j + 1].create(alphaPyrs[i][j + 1].size(), CV_16SC1);
                scaledSet16SC1Mask32SC1(tempAlphaPyr[j + 1], 256, alphaPyrs[i][j + 1]);
                pyramidDown16SC1To16SC1(weightPyrs[i][j], weightPyrs[i][j + 1], cv::Size(), true);
            }
        }

        /* :606-615: level sizes and the result pyramid */
        std::vector<cv::Size> sizes(numLevels + 1);
        sizes[0] = cv::Size(cols, rows);
        for (int i = 1; i <= numLevels; i++)
            sizes[i] = cv::Size((sizes[i - 1].width + 1) / 2, (sizes[i - 1].height + 1) / 2);
        std::vector<cv::cuda::GpuMat> resultPyr(numLevels + 1), imageUpPyr(numLevels + 1),
            resultUpPyr(numLevels + 1);
        for (int i = 0; i <= numLevels; i++) resultPyr[i].create(sizes[i], CV_32SC4);

        /* :617-638: fullMask, resultWeightPyr, maskNot */
        cv::Mat mask = cv::Mat::zeros(rows, cols, CV_8UC1);
        for (int i = 0; i < numImages; i++)
            for (size_t p = 0; p < px; ++p) mask.data[p] |= masks[px * i + p];
        size_t nonZero = 0;
        for (size_t p = 0; p < px; ++p) nonZero += mask.data[p] != 0;
        const bool fullMask = nonZero == px;
        std::vector<cv::cuda::GpuMat> resultWeightPyr;
        cv::cuda::GpuMat maskNot;
        if (!fullMask) {
            resultWeightPyr.resize(numLevels + 1);
            for (int i = 0; i < numLevels + 1; i++) {
                resultWeightPyr[i].create(sizes[i], CV_32SC1);
                resultWeightPyr[i].setTo(0);
            }
            for (int i = 0; i < numImages; i++)
                for (int j = 0; j <= numLevels; j++) accumulate16SC1To32SC1(weightPyrs[i][j], resultWeightPyr[j]);
            for (size_t p = 0; p < px; ++p) mask.data[p] = (uint8_t)~mask.data[p];
            maskNot.upload(mask);
        }

        /* blend: :785-823 */
        for (int i = 0; i <= numLevels; i++) resultPyr[i].setTo(0);
        std::vector<cv::cuda::GpuMat> imagePyr(numLevels + 1);
        for (int i = 0; i < numImages; i++) {
            cv::cuda::GpuMat image(copyIn(images + px * 4 * i, rows, cols, CV_16SC4));
            image.copyTo(imagePyr[0]);
            for (int j = 0; j < numLevels; j++)
                pyramidDown16SC4To16SC4(imagePyr[j], alphaPyrs[i][j + 1], imagePyr[j + 1], true);
            for (int j = 0; j < numLevels; j++) {
                pyramidUp16SC4To16SC4(imagePyr[j + 1], imageUpPyr[j], imagePyr[j].size(), true);
                subtract16SC4(imagePyr[j], imageUpPyr[j], imagePyr[j]);
            }
            for (int j = 0; j <= numLevels; j++) accumulate16SC4To32SC4(imagePyr[j], weightPyrs[i][j], resultPyr[j]);
        }
        if (fullMask)
            for (int j = 0; j <= numLevels; j++) normalize32SC4(resultPyr[j]);
        else
            for (int j = 0; j <= numLevels; j++) normalize32SC4(resultPyr[j], resultWeightPyr[j]);
        if (norm) {
            int32_t* o = norm;
            for (int j = 0; j <= numLevels; j++) {
                copyOut(resultPyr[j], o);
                o += (size_t)sizes[j].area() * 4;
            }
        }
        /* restoreImageFromLaplacePyramid (:220-231) */
        for (size_t i = resultPyr.size() - 1; i > 0; --i) {
            pyramidUp32SC4To32SC4(resultPyr[i], resultUpPyr[i - 1], resultPyr[i - 1].size(), true);
            add32SC4(resultUpPyr[i - 1], resultPyr[i - 1], resultPyr[i - 1]);
        }
        cv::cuda::GpuMat blendImage;
        resultPyr[0].convertTo(blendImage, CV_8U);
        if (!fullMask) blendImage.setTo(0, maskNot);
        copyOut(blendImage, blend);

        if (coll) {
            int32_t* o = coll;
            for (int j = 0; j <= numLevels; j++) {
                copyOut(resultPyr[j], o);
                o += (size_t)sizes[j].area() * 4;
            }
        }
        const size_t lp = levelPixels(W, H, numLevels);
        for (int i = 0; i < numImages; i++) {
            size_t off = 0;
            for (int j = 0; j <= numLevels; j++) {
                if (weights) copyOut(weightPyrs[i][j], weights + lp * i + off);
                if (alphas) {
                    if (j == 0) std::memset(alphas + lp * i, 0, px * sizeof(int32_t));
                    else copyOut(alphaPyrs[i][j], alphas + lp * i + off);
                }
                off += (size_t)sizes[j].area();
            }
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

/* cvtBGR32ToYUV420P / cvtBGR32ToNV12 (source/CudaAccel/ImageProc.cu:126-162).
   fmt 420: planes y (W*H), u and v (W/2*H/2); fmt 12: y and uv (W*H/2). */
int psref_bgr32_to_yuv(const uint8_t* bgr, int W, int H, int fmt, uint8_t* y, uint8_t* u, uint8_t* v)
{
    try {
        cv::cuda::GpuMat src(copyIn(bgr, H, W, CV_8UC4)), gy, gu, gv;
        if (fmt == 420) {
            cvtBGR32ToYUV420P(src, gy, gu, gv);
            copyOut(gy, y);
            copyOut(gu, u);
            copyOut(gv, v);
        } else {
            cvtBGR32ToNV12(src, gy, gu);
            copyOut(gy, y);
            copyOut(gu, u);
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

/* cvtYUV420PToBGR32 / cvtNV12ToBGR32 (source/CudaAccel/ImageProc.cu:224-259). */
int psref_yuv_to_bgr32(const uint8_t* y, const uint8_t* u, const uint8_t* v, int W, int H, int fmt, uint8_t* bgr)
{
    try {
        cv::cuda::GpuMat gy(copyIn(y, H, W, CV_8UC1)), out;
        if (fmt == 420) {
            cv::cuda::GpuMat gu(copyIn(u, H / 2, W / 2, CV_8UC1)), gv(copyIn(v, H / 2, W / 2, CV_8UC1));
            cvtYUV420PToBGR32(gy, gu, gv, out);
        } else {
            cv::cuda::GpuMat guv(copyIn(u, H / 2, W, CV_8UC1));
            cvtNV12ToBGR32(gy, guv, out);
        }
        copyOut(out, bgr);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

}  /* extern "C" */
