/* cv::cuda::StreamAccessor for the reference build of the checker (TEST
   INFRASTRUCTURE ONLY): every stream is the emulated null stream. */
#ifndef PSEMU_OPENCV2_CUDA_STREAM_ACCESSOR_HPP
#define PSEMU_OPENCV2_CUDA_STREAM_ACCESSOR_HPP

#include "cuda_runtime.h"
#include "opencv2/core/cuda.hpp"

namespace cv {
namespace cuda {
struct StreamAccessor {
    static cudaStream_t getStream(const Stream&) { return nullptr; }
};
}  // namespace cuda
}  // namespace cv

#endif
