/* cv::cuda::device::divUp and cudaSafeCall for the reference build of the
   checker (TEST INFRASTRUCTURE ONLY). */
#ifndef PSEMU_OPENCV2_CUDA_COMMON_HPP
#define PSEMU_OPENCV2_CUDA_COMMON_HPP

#include <stdexcept>

#include "cuda_runtime.h"
#include "opencv2/core.hpp"

namespace cv {
namespace cuda {
namespace device {
inline int divUp(int total, int grain) { return (total + grain - 1) / grain; }
}  // namespace device
}  // namespace cuda
}  // namespace cv

#define cudaSafeCall(expr) \
    do { if ((expr) != cudaSuccess) throw std::runtime_error("cudaSafeCall: " #expr); } while (0)

#endif
