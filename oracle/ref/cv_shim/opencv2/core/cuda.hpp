/*
 * opencv2/core/cuda.hpp -- cv::cuda::GpuMat and cv::cuda::Stream for the
 * reference build of the checker (TEST INFRASTRUCTURE ONLY).
 *
 * The reference's kernels run on host cores under cuda_emu, so "device"
 * memory is host memory: a GpuMat is a Mat with OpenCV's GpuMat method
 * names (upload, download, and setTo / copyTo / convertTo / clone taking and
 * returning GpuMat).  Rows are packed rather than pitched; the kernels take
 * the step as an argument, so the layout does not change what they compute.
 */
#ifndef PSEMU_OPENCV2_CORE_CUDA_HPP
#define PSEMU_OPENCV2_CORE_CUDA_HPP

#include "opencv2/core.hpp"

namespace cv {
namespace cuda {

class GpuMat : public Mat {
public:
    GpuMat() {}
    GpuMat(int r, int c, int type) : Mat(r, c, type) {}
    GpuMat(Size s, int type) : Mat(s, type) {}
    GpuMat(int r, int c, int type, void* ptr, size_t st = 0) : Mat(r, c, type, ptr, st) {}
    GpuMat(Size s, int type, void* ptr, size_t st = 0) : Mat(s, type, ptr, st) {}
    explicit GpuMat(const Mat& m) : Mat(m) {}

    void upload(const Mat& m) { m.copyTo(*this); }
    void download(Mat& m) const { Mat::copyTo(m); }
    GpuMat& setTo(const Scalar& s, const GpuMat& mask = GpuMat())
    {
        Mat::setTo(s, mask);
        return *this;
    }
    void copyTo(GpuMat& dst) const { Mat::copyTo(dst); }
    GpuMat clone() const
    {
        GpuMat g;
        Mat::copyTo(g);
        return g;
    }
    void convertTo(GpuMat& dst, int rtype) const
    {
        Mat out;
        Mat::convertTo(out, rtype);
        dst = GpuMat(out);
    }
};

class Stream {
public:
    static Stream& Null()
    {
        static Stream s;
        return s;
    }
};

}  // namespace cuda
}  // namespace cv

#endif
