/*
 * opencv2/highgui.hpp -- TEST INFRASTRUCTURE ONLY.  Declarations of the
 * display and file calls that the reference's debugging helpers name; the
 * oracle's pin never calls them, and oracle/ref/ref_driver.cpp defines them
 * to throw.
 */
#ifndef PSEMU_OPENCV2_HIGHGUI_HPP
#define PSEMU_OPENCV2_HIGHGUI_HPP
#include <string>
#include "opencv2/core.hpp"
namespace cv {
void imshow(const std::string& name, const Mat& m);
int waitKey(int delay = 0);
bool imwrite(const std::string& path, const Mat& m);
}
#endif
