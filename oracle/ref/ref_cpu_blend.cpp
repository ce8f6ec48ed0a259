/*
 * ref_cpu_blend.cpp -- C entry point over the reference's CPU multiband
 * blend, for pinning oracle/ps_oracle_cpu.c against it.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile's `ref` target compiles
 * source/Blend/MultiBandBlend.cpp and source/Blend/Pyramid.cpp unchanged,
 * from the reference tree where they lie, against the OpenCV subset in
 * cv_shim/, and links them with this file into oracle/_ref/libpsref.so.
 * psref_cpu_mb_blend below runs the reference's own class,
 * TilingMultibandBlendFast: prepare (MultiBandBlend.cpp:906-985), then
 * blend (:987-1031).
 *
 * The blender keeps its pyramids private; the pin reads them after a blend,
 * so its header is included with private members made public (the layout
 * does not change).  The unique masks are given, as in the CudaAccel pin:
 * getNonIntersectingMasks (source/Blend/Mask.cpp) needs OpenCV's
 * distanceTransform, so the definition below returns the masks the caller
 * passed.  The other functions that MultiBandBlend.cpp names but that the
 * pinned class never calls (the aux-buffer pyramids of Pyramid3.cpp, the
 * checks of Prepare.cpp, highgui) are defined to throw.
 */
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "opencv2/core.hpp"
#include "opencv2/highgui.hpp"

#define private public
#include "ZBlend.h"
#undef private
#include "ZBlendAlgo.h"

namespace {
thread_local const std::vector<cv::Mat>* g_givenUniqueMasks = nullptr;

[[noreturn]] void notOnPinnedPath(const char* what)
{
    throw std::runtime_error(std::string(what) + " is not on the pinned path");
}
}  // namespace

void getNonIntersectingMasks(const std::vector<cv::Mat>& masks, std::vector<cv::Mat>& uniqueMasks)
{
    if (!g_givenUniqueMasks || g_givenUniqueMasks->size() != masks.size())
        throw std::runtime_error("getNonIntersectingMasks: no unique masks given");
    uniqueMasks.resize(masks.size());
    for (size_t i = 0; i < masks.size(); ++i) uniqueMasks[i] = (*g_givenUniqueMasks)[i].clone();
}

bool checkType(const std::vector<cv::Mat>&, int) { notOnPinnedPath("checkType"); }
bool checkSize(const std::vector<cv::Mat>&) { notOnPinnedPath("checkSize"); }
void pyramidDownTo32S(const cv::Mat&, cv::Mat&, std::vector<unsigned char>&, std::vector<unsigned char>&,
                      const cv::Size&, int, int)
{
    notOnPinnedPath("pyramidDownTo32S with row buffers");
}
void pyramidUp(const cv::Mat&, cv::Mat&, std::vector<unsigned char>&, std::vector<unsigned char>&, const cv::Size&,
               int, int)
{
    notOnPinnedPath("pyramidUp with row buffers");
}
namespace cv {
void imshow(const std::string&, const Mat&) { notOnPinnedPath("imshow"); }
int waitKey(int) { notOnPinnedPath("waitKey"); }
bool imwrite(const std::string&, const Mat&) { notOnPinnedPath("imwrite"); }
}  // namespace cv

extern "C" {

/* TilingMultibandBlendFast::prepare(masks, maxLevels, minLength) then
   ::blend(images, blendImage).  Inputs: n coverage masks and n unique
   masks (W*H bytes each, 0 / non-zero) and n level-0 images of W*H int16x4
   (channels B, G, R are passed as the reference's CV_16SC3 images).
   Outputs (nullable except blend): blend W*H*4 bytes (B, G, R, 0); coll the
   collapsed result pyramid, int32x3, levels 0..L packed; weights and alphas
   the n weight (int16) and alpha (int32, level 0 zero) pyramids, levels
   0..L packed; levels_out the number of levels.  Returns 0, or -1 when the
   reference raised an error or prepare failed. */
int psref_cpu_mb_blend(int n, int W, int H, int maxLevels, int minLength, const uint8_t* masks, const uint8_t* uniq,
                       const int16_t* images, uint8_t* blend, int32_t* coll, int16_t* weights, int32_t* alphas,
                       int* levels_out)
{
    try {
        const size_t px = (size_t)W * H;
        std::vector<cv::Mat> m(n), u(n), imgs(n);
        for (int i = 0; i < n; ++i) {
            m[i].create(H, W, CV_8UC1);
            std::memcpy(m[i].data, masks + px * i, px);
            u[i].create(H, W, CV_8UC1);
            std::memcpy(u[i].data, uniq + px * i, px);
            imgs[i].create(H, W, CV_16SC3);
            const int16_t* s = images + px * 4 * i;
            short* d = imgs[i].ptr<short>(0);
            for (size_t p = 0; p < px; ++p)
                for (int c = 0; c < 3; ++c) d[3 * p + c] = s[4 * p + c];
        }
        TilingMultibandBlendFast b;
        g_givenUniqueMasks = &u;
        const bool ok = b.prepare(m, maxLevels, minLength);
        g_givenUniqueMasks = nullptr;
        if (!ok) return -1;
        cv::Mat out;
        b.blend(imgs, out);
        for (size_t p = 0; p < px; ++p) {
            for (int c = 0; c < 3; ++c) blend[4 * p + c] = out.data[3 * p + c];
            blend[4 * p + 3] = 0;
        }
        const int L = b.numLevels;
        if (levels_out) *levels_out = L;
        size_t lp = 0;
        for (int j = 0; j <= L; ++j) lp += (size_t)b.resultPyr[j].rows * b.resultPyr[j].cols;
        if (coll) {
            int32_t* o = coll;
            for (int j = 0; j <= L; ++j) {
                const size_t k = (size_t)b.resultPyr[j].rows * b.resultPyr[j].cols * 3;
                std::memcpy(o, b.resultPyr[j].data, k * sizeof(int32_t));
                o += k;
            }
        }
        for (int i = 0; i < n; ++i) {
            size_t off = 0;
            for (int j = 0; j <= L; ++j) {
                const size_t k = (size_t)b.resultPyr[j].rows * b.resultPyr[j].cols;
                if (weights) std::memcpy(weights + lp * i + off, b.weightPyrs[i][j].data, k * sizeof(int16_t));
                if (alphas) {
                    if (j == 0) std::memset(alphas + lp * i, 0, k * sizeof(int32_t));
                    else std::memcpy(alphas + lp * i + off, b.alphaPyrs[i][j].data, k * sizeof(int32_t));
                }
                off += k;
            }
        }
        return 0;
    } catch (const std::exception&) {
        g_givenUniqueMasks = nullptr;
        return -1;
    }
}

}  /* extern "C" */
