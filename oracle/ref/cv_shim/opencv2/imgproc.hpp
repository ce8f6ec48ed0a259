/*
 * opencv2/imgproc.hpp -- TEST INFRASTRUCTURE ONLY.  The reference's CPU blend
 * includes this header but, on the functions the oracle's pin compiles,
 * uses only core.hpp's subset.
 */
#ifndef PSEMU_OPENCV2_IMGPROC_HPP
#define PSEMU_OPENCV2_IMGPROC_HPP
#include "opencv2/core.hpp"
#endif
