// panostitch.hpp -- C++ facade over the C ABI with the reference's class and
// method names (source/Task/RicohUtil.h:193-220,
// source/CudaAccel/CudaInterface.h:45-82), so Task-layer call sites switch
// by changing a type.  Header-only; link with -lpanostitch.
//
// Differences from the reference signatures, all forced by OpenCV being
// absent: images are ps_image views instead of cv::Mat / cv::cuda::GpuMat,
// camera parameters are passed directly instead of a file path, sizes are
// panostitch::Size.  Errors return false and keep the message in
// lastError(), as the reference returns false after lprintf.
#pragma once

#include <cstdio>
#include <string>
#include <vector>

#include "panostitch.h"

namespace panostitch {

struct Size {
    int width = 0, height = 0;
};

class CudaPanoramaRender2 {
public:
    CudaPanoramaRender2() { ps_render_create(&r_); }
    ~CudaPanoramaRender2() { ps_render_destroy(r_); }
    CudaPanoramaRender2(const CudaPanoramaRender2&) = delete;
    CudaPanoramaRender2& operator=(const CudaPanoramaRender2&) = delete;

    // CudaPanoramaRender2::prepare (source/Task/RicohUtil.cpp:1091-1205)
    bool prepare(const std::vector<ps_photo_param>& params, int highQualityBlend, int blendParam,
                 const Size& srcSize, const Size& dstSize, void* stream = nullptr)
    {
        return ok(ps_render_prepare(r_, params.data(), (int)params.size(), highQualityBlend, blendParam,
                                    srcSize.width, srcSize.height, dstSize.width, dstSize.height, stream));
    }

    // CudaPanoramaRender2::prepare(path, ...) with a PTGui .pts camera file
    bool prepare(const std::string& path, int highQualityBlend, int blendParam, const Size& srcSize,
                 const Size& dstSize, void* stream = nullptr)
    {
        return ok(ps_render_prepare_file(r_, path.c_str(), highQualityBlend, blendParam, srcSize.width, srcSize.height,
                                         dstSize.width, dstSize.height, stream));
    }

    // CudaPanoramaRender2::render (source/Task/RicohUtil.cpp:1207-1339).  Like
    // the reference, LUTs that are not numImages x 3 x 256 are skipped with a
    // warning (:1239-1265) instead of failing the frame.
    bool render(const std::vector<ps_image>& src, ps_image& dst,
                const std::vector<std::vector<std::vector<unsigned char>>>& luts = {}, void* stream = nullptr)
    {
        std::vector<unsigned char> flat;
        const bool correct = flattenLuts(luts, flat);
        return ok(ps_render_render(r_, src.data(), (int)src.size(), correct ? flat.data() : nullptr,
                                   correct ? getNumImages() : 0, &dst, stream));
    }

    // render followed by the encoder handoff (cvtBGR32ToYUV420P / cvtBGR32ToNV12
    // and the planes' download, source/Task/PanoramaLocalDiskTask.cpp:2054-2076)
    bool renderYuv(const std::vector<ps_image>& src, const ps_planar_image& dst,
                   const std::vector<std::vector<std::vector<unsigned char>>>& luts = {}, void* stream = nullptr)
    {
        std::vector<unsigned char> flat;
        const bool correct = flattenLuts(luts, flat);
        return ok(ps_render_render_yuv(r_, src.data(), (int)src.size(), correct ? flat.data() : nullptr,
                                       correct ? getNumImages() : 0, &dst, stream));
    }

    // render from decoder frames (YUV420P / NV12, host or device): the
    // device converts them as cvtYUV420PToBGR32 / cvtNV12ToBGR32 do
    // (source/CudaAccel/ImageProc.cu:165-259); out to a BGR canvas, or with
    // the encoder handoff to planes (ydst)
    bool renderPlanar(const std::vector<ps_planar_image>& src, ps_image* dst, const ps_planar_image* ydst,
                      const std::vector<std::vector<std::vector<unsigned char>>>& luts = {}, void* stream = nullptr)
    {
        std::vector<unsigned char> flat;
        const bool correct = flattenLuts(luts, flat);
        return ok(ps_render_render_planar(r_, src.data(), (int)src.size(), correct ? flat.data() : nullptr,
                                          correct ? getNumImages() : 0, dst, ydst, stream));
    }

    // The custom masks of the frame's interval (one host uint8 dstSize mask per
    // camera: its custom mask, or its unique mask where it has none), as the
    // Tasks pass them to CudaTilingMultibandBlendFast::blend(images, masks,
    // blendImage) (source/Task/PanoramaPreviewTask.cpp:382-400); an empty
    // vector returns to the unique masks.  Call when the interval changes.
    bool setCustomMasks(const std::vector<const uint8_t*>& masks, void* stream = nullptr)
    {
        return ok(ps_render_set_custom_masks(r_, masks.empty() ? nullptr : masks.data(), (int)masks.size(), stream));
    }

    void clear() { ps_render_clear(r_); }
    int getNumImages() const { return ps_render_get_num_images(r_); }
    const std::string& lastError() const { return err_; }
    ps_render* handle() const { return r_; }

private:
    bool ok(int status)
    {
        if (status == PS_OK) return true;
        err_ = ps_last_error();
        return false;
    }
    // The reference's LUT check (source/Task/RicohUtil.cpp:1239-1265): a
    // malformed non-empty set is skipped with a warning.
    bool flattenLuts(const std::vector<std::vector<std::vector<unsigned char>>>& luts,
                     std::vector<unsigned char>& flat) const
    {
        const int n = getNumImages();
        bool correct = (int)luts.size() == n && n > 0;
        for (size_t i = 0; correct && i < luts.size(); i++) {
            if (luts[i].size() != 3) correct = false;
            for (size_t c = 0; correct && c < luts[i].size(); c++)
                if (luts[i][c].size() != 256) correct = false;
        }
        if (!correct && !luts.empty())
            std::fprintf(stderr, "Warning in render, the non-empty look up tables not satisfied, skip correction\n");
        if (correct) {
            flat.reserve((size_t)n * 768);
            for (const auto& cam : luts)
                for (const auto& ch : cam) flat.insert(flat.end(), ch.begin(), ch.end());
        }
        return correct;
    }
    ps_render* r_ = nullptr;
    std::string err_;
};

// CudaRicohPanoramaRender (source/Task/RicohUtil.cpp:1363-1406): a dual
// fisheye camera that delivers both lenses in one frame.  The rig has two
// cameras whose crops select the halves of that frame; render takes the one
// frame and stitches it as both cameras' source (the library uploads a host
// frame that appears twice only once).  getNumImages is 1.
class CudaRicohPanoramaRender {
public:
    bool prepare(const std::vector<ps_photo_param>& params, int highQualityBlend, int blendParam,
                 const Size& srcSize, const Size& dstSize, void* stream = nullptr)
    {
        return checked(r_.prepare(params, highQualityBlend, blendParam, srcSize, dstSize, stream));
    }
    bool prepare(const std::string& path, int highQualityBlend, int blendParam, const Size& srcSize,
                 const Size& dstSize, void* stream = nullptr)
    {
        return checked(r_.prepare(path, highQualityBlend, blendParam, srcSize, dstSize, stream));
    }
    bool render(const std::vector<ps_image>& src, ps_image& dst,
                const std::vector<std::vector<std::vector<unsigned char>>>& luts = {}, void* stream = nullptr)
    {
        if (r_.getNumImages() != 2) {
            err_ = "have not prepared or prepare failed before";
            return false;
        }
        if (src.size() != 1) {
            err_ = "src size = " + std::to_string(src.size()) + ", requires 1";
            return false;
        }
        const std::vector<ps_image> both(2, src[0]);
        if (r_.render(both, dst, luts, stream)) return true;
        err_ = r_.lastError();
        return false;
    }
    void clear() { r_.clear(); }
    int getNumImages() const { return r_.getNumImages() == 2 ? 1 : 0; }
    const std::string& lastError() const { return err_; }
    ps_render* handle() const { return r_.handle(); }

private:
    // RicohUtil.cpp:1368-1373: the prepared rig must have two cameras
    bool checked(bool prepared)
    {
        if (!prepared) {
            err_ = r_.lastError();
            return false;
        }
        if (r_.getNumImages() != 2) {
            err_ = "num images = " + std::to_string(r_.getNumImages()) + ", requires 2";
            r_.clear();
            return false;
        }
        return true;
    }
    CudaPanoramaRender2 r_;
    std::string err_;
};

// CudaTilingMultibandBlendFast (source/CudaAccel/CudaInterface.h:45-82)
class CudaTilingMultibandBlendFast {
public:
    CudaTilingMultibandBlendFast() { ps_blender_create(&b_); }
    ~CudaTilingMultibandBlendFast() { ps_blender_destroy(b_); }
    CudaTilingMultibandBlendFast(const CudaTilingMultibandBlendFast&) = delete;
    CudaTilingMultibandBlendFast& operator=(const CudaTilingMultibandBlendFast&) = delete;

    // prepare(masks, maxLevels, minLength); seams replace getNonIntersectingMasks
    bool prepare(const std::vector<const uint8_t*>& masks, const std::vector<const uint8_t*>& seams, int width,
                 int height, int maxLevels, int minLength, void* stream = nullptr)
    {
        if (masks.size() != seams.size()) {
            err_ = "masks and seams differ in count";
            return false;
        }
        return ok(ps_blender_prepare(b_, masks.data(), seams.data(), (int)masks.size(), width, height, maxLevels,
                                     minLength, stream));
    }
    // blend(images, blendImage): device CV_16SC4 (format 16) or CV_8UC4 (8) images
    bool blend(const std::vector<const void*>& images, const std::vector<long long>& pitches, int format,
               ps_image& dst, void* stream = nullptr)
    {
        return ok(ps_blender_blend(b_, images.data(), pitches.data(), format, &dst, stream));
    }
    // begin / tile(image, index) / end(blendImage) (CudaMultibandBlend.cpp:737-783):
    // the blend fed one camera at a time
    bool begin(void* stream = nullptr) { return ok(ps_blender_begin(b_, stream)); }
    bool tile(const void* image, long long pitch, int format, int index, void* stream = nullptr)
    {
        return ok(ps_blender_tile(b_, image, pitch, format, index, stream));
    }
    bool end(ps_image& dst, void* stream = nullptr) { return ok(ps_blender_end(b_, &dst, stream)); }
    // getUniqueMasks (:895-901): into host buffers of width * height bytes
    bool getUniqueMasks(const std::vector<uint8_t*>& masks)
    {
        return ok(ps_blender_get_unique_masks(b_, masks.data(), (int)masks.size()));
    }
    // calcUsedMemorySize (:903-920) and estimateMemorySize (:922-926)
    long long calcUsedMemorySize() const { return ps_blender_used_memory(b_); }
    static long long estimateMemorySize(int width, int height, int numImages, int maxLevels = 16)
    {
        return ps_blender_estimate_memory(width, height, numImages, maxLevels);
    }
    int numLevels() const { return ps_blender_get_num_levels(b_); }
    const std::string& lastError() const { return err_; }

private:
    bool ok(int status)
    {
        if (status == PS_OK) return true;
        err_ = ps_last_error();
        return false;
    }
    ps_blender* b_ = nullptr;
    std::string err_;
};

}  // namespace panostitch
