/*
 * opencv2/core.hpp -- the subset of OpenCV 3.0's core API that the
 * reference's geometry, remap and pyramid sources use, so that they compile
 * unchanged without OpenCV.
 *
 * TEST INFRASTRUCTURE ONLY: part of the recipe that builds the reference's
 * own code into oracle/_ref/ as the checker's pin.  Written for this
 * project from OpenCV's documented behaviour; the arithmetic that the
 * reference takes from OpenCV is:
 *   - saturate_cast<T>(floating v): round to nearest, ties to even (cvRound
 *     as OpenCV's SSE2 build computes it on the reference's x64 target),
 *     then clamp to T's range; saturate_cast<T>(integer v): clamp;
 *   - Mat::convertTo(dst, depth): saturate_cast<dst depth> per element
 *     (alpha = 1, beta = 0 only);
 *   - Mat::setTo(s, mask): every channel of the elements whose mask byte is
 *     non-zero (all elements without a mask) takes saturate_cast(s[c]);
 *   - add / subtract: saturate_cast<depth>(a +- b) per element, where the
 *     sum is formed in int for the integer depths (so 32-bit sums wrap);
 *   - bitwise operators on 8-bit masks, countNonZero;
 *   - borderInterpolate: OpenCV's documented mapping of an outside index p
 *     (reflect-101 and reflect mirror about the edge, with or without
 *     repeating it, and map every index to 0 when len == 1; wrap takes p
 *     modulo len; replicate clamps).
 * Images are continuous: step = cols * elemSize, so rows are packed.
 */
#ifndef PSEMU_OPENCV2_CORE_HPP
#define PSEMU_OPENCV2_CORE_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <ostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_MAT_DEPTH_MASK 7
#define CV_MAT_DEPTH(t) ((t) & CV_MAT_DEPTH_MASK)
#define CV_MAT_CN(t) ((((t) >> CV_CN_SHIFT) & 511) + 1)
#define CV_MAKETYPE(depth, cn) (CV_MAT_DEPTH(depth) + (((cn) - 1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC2 CV_MAKETYPE(CV_8U, 2)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_8UC4 CV_MAKETYPE(CV_8U, 4)
#define CV_16SC1 CV_MAKETYPE(CV_16S, 1)
#define CV_16SC2 CV_MAKETYPE(CV_16S, 2)
#define CV_16SC3 CV_MAKETYPE(CV_16S, 3)
#define CV_16SC4 CV_MAKETYPE(CV_16S, 4)
#define CV_32SC1 CV_MAKETYPE(CV_32S, 1)
#define CV_32SC2 CV_MAKETYPE(CV_32S, 2)
#define CV_32SC3 CV_MAKETYPE(CV_32S, 3)
#define CV_32SC4 CV_MAKETYPE(CV_32S, 4)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)
#define CV_32FC2 CV_MAKETYPE(CV_32F, 2)
#define CV_32FC3 CV_MAKETYPE(CV_32F, 3)
#define CV_32FC4 CV_MAKETYPE(CV_32F, 4)
#define CV_64FC1 CV_MAKETYPE(CV_64F, 1)
#define CV_64FC2 CV_MAKETYPE(CV_64F, 2)

#define CV_CN_MAX 512
#define CV_CPU_SSE 1
#define CV_CPU_SSE2 2
#define CV_StsUnsupportedFormat (-210)
#define CV_Error(code, msg) throw std::runtime_error(std::string("CV_Error: ") + (msg))

#define CV_Assert(expr) \
    do { if (!(expr)) throw std::runtime_error(std::string("CV_Assert failed: ") + #expr); } while (0)

typedef unsigned char uchar;
typedef signed char schar;
typedef unsigned short ushort;

/* MSVC's bounded sprintf into a char array, which the reference's
   debugging helpers call. */
template <size_t N, class... A> inline int sprintf_s(char (&buf)[N], const char* fmt, A... a)
{
    return std::snprintf(buf, N, fmt, a...);
}

namespace cv {

typedef unsigned char uchar;
typedef signed char schar;
typedef unsigned short ushort;

inline int cvRound(double v) { return (int)std::nearbyint(v); }

enum { BORDER_CONSTANT = 0, BORDER_REPLICATE = 1, BORDER_REFLECT = 2, BORDER_WRAP = 3, BORDER_REFLECT_101 = 4,
       BORDER_REFLECT101 = 4, BORDER_DEFAULT = 4 };

inline int borderInterpolate(int p, int len, int borderType)
{
    if (p >= 0 && p < len) return p;
    switch (borderType) {
    case BORDER_REPLICATE: return p < 0 ? 0 : len - 1;
    case BORDER_REFLECT:
    case BORDER_REFLECT_101: {
        const int skipEdge = borderType == BORDER_REFLECT_101;
        if (len == 1) return 0;
        while (p < 0 || p >= len) p = p < 0 ? -p - 1 + skipEdge : 2 * len - 1 - p - skipEdge;
        return p;
    }
    case BORDER_WRAP:
        if (len <= 0) throw std::runtime_error("borderInterpolate: empty range");
        p %= len;
        return p < 0 ? p + len : p;
    default: return -1;
    }
}

inline bool checkHardwareSupport(int) { return true; }
inline size_t alignSize(size_t sz, int n) { return (sz + n - 1) & ~(size_t)(n - 1); }
template <class T> inline T* alignPtr(T* p, int n) { return (T*)(((size_t)p + n - 1) & ~(size_t)(n - 1)); }

/* Heap buffer of n elements (value-initialised). */
template <class T, size_t = 0> class AutoBuffer {
public:
    explicit AutoBuffer(size_t n) : v_(n ? n : 1) {}
    operator T*() { return v_.data(); }
    operator const T*() const { return v_.data(); }
private:
    std::vector<T> v_;
};

template <class T> inline T saturate_cast(int v)
{
    if (std::numeric_limits<T>::is_integer) {
        if (v < (int)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
        if (v > (int)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
    }
    return (T)v;
}
template <> inline int saturate_cast<int>(int v) { return v; }
template <> inline float saturate_cast<float>(int v) { return (float)v; }
template <> inline double saturate_cast<double>(int v) { return (double)v; }
template <class T> inline T saturate_cast(double v)
{
    if (std::numeric_limits<T>::is_integer) {
        const double r = std::nearbyint(v);
        if (r < (double)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
        if (r > (double)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
        return (T)r;
    }
    return (T)v;
}
template <class T> inline T saturate_cast(float v) { return saturate_cast<T>((double)v); }
template <> inline float saturate_cast<float>(float v) { return v; }
template <class T> inline T saturate_cast(uchar v) { return saturate_cast<T>((int)v); }
template <class T> inline T saturate_cast(schar v) { return saturate_cast<T>((int)v); }
template <class T> inline T saturate_cast(short v) { return saturate_cast<T>((int)v); }
template <class T> inline T saturate_cast(ushort v) { return saturate_cast<T>((int)v); }

struct Size {
    int width = 0, height = 0;
    Size() {}
    Size(int w, int h) : width(w), height(h) {}
    int area() const { return width * height; }
    bool operator==(const Size& o) const { return width == o.width && height == o.height; }
    bool operator!=(const Size& o) const { return !(*this == o); }
};

template <class T> struct Point_ {
    T x, y;
    Point_() : x(0), y(0) {}
    Point_(T vx, T vy) : x(vx), y(vy) {}
};
typedef Point_<int> Point;
typedef Point_<float> Point2f;
typedef Point_<double> Point2d;

template <class T, int n> struct Vec {
    T val[n];
    T& operator[](int i) { return val[i]; }
    const T& operator[](int i) const { return val[i]; }
};
typedef Vec<uchar, 3> Vec3b;
typedef Vec<uchar, 4> Vec4b;
typedef Vec<short, 3> Vec3s;
typedef Vec<short, 4> Vec4s;
typedef Vec<int, 4> Vec4i;
typedef Vec<float, 3> Vec3f;
typedef Vec<float, 4> Vec4f;
typedef Vec<double, 2> Vec2d;
typedef Vec<double, 3> Vec3d;

template <class T> struct Rect_ {
    T x = 0, y = 0, width = 0, height = 0;
    Rect_() {}
    Rect_(T vx, T vy, T w, T h) : x(vx), y(vy), width(w), height(h) {}
    Size size() const { return Size((int)width, (int)height); }
    T area() const { return width * height; }
};
typedef Rect_<int> Rect;
template <class T> inline bool operator==(const Rect_<T>& a, const Rect_<T>& b)
{
    return a.x == b.x && a.y == b.y && a.width == b.width && a.height == b.height;
}
template <class T> inline Rect_<T> operator&(const Rect_<T>& a, const Rect_<T>& b)
{
    const T x0 = std::max(a.x, b.x), y0 = std::max(a.y, b.y);
    const T x1 = std::min(a.x + a.width, b.x + b.width), y1 = std::min(a.y + a.height, b.y + b.height);
    if (x1 <= x0 || y1 <= y0) return Rect_<T>();
    return Rect_<T>(x0, y0, x1 - x0, y1 - y0);
}

struct Range {
    int start = 0, end = 0;
    Range() {}
    Range(int s, int e) : start(s), end(e) {}
};

struct Scalar {
    double val[4];
    Scalar(double v0 = 0, double v1 = 0, double v2 = 0, double v3 = 0) : val{v0, v1, v2, v3} {}
    static Scalar all(double v) { return Scalar(v, v, v, v); }
};

inline size_t depthSize(int depth)
{
    static const size_t s[] = {1, 1, 2, 2, 4, 4, 8, 0};
    return s[depth & 7];
}

/* Element-wise helpers shared by Mat and cuda::GpuMat. */
namespace detail {
template <class S, class D> inline void convertRow(const S* s, D* d, size_t n)
{
    for (size_t i = 0; i < n; ++i) d[i] = saturate_cast<D>(s[i]);
}
template <class S> inline void convertRowTo(const S* s, void* d, int ddepth, size_t n)
{
    switch (ddepth) {
    case CV_8U: convertRow(s, (uchar*)d, n); break;
    case CV_8S: convertRow(s, (schar*)d, n); break;
    case CV_16U: convertRow(s, (ushort*)d, n); break;
    case CV_16S: convertRow(s, (short*)d, n); break;
    case CV_32S: convertRow(s, (int*)d, n); break;
    case CV_32F: convertRow(s, (float*)d, n); break;
    case CV_64F: convertRow(s, (double*)d, n); break;
    }
}
inline void convertAny(const void* s, int sdepth, void* d, int ddepth, size_t n)
{
    switch (sdepth) {
    case CV_8U: convertRowTo((const uchar*)s, d, ddepth, n); break;
    case CV_8S: convertRowTo((const schar*)s, d, ddepth, n); break;
    case CV_16U: convertRowTo((const ushort*)s, d, ddepth, n); break;
    case CV_16S: convertRowTo((const short*)s, d, ddepth, n); break;
    case CV_32S: convertRowTo((const int*)s, d, ddepth, n); break;
    case CV_32F: convertRowTo((const float*)s, d, ddepth, n); break;
    case CV_64F: convertRowTo((const double*)s, d, ddepth, n); break;
    }
}
inline void setElem(uchar* p, int type, const Scalar& s)
{
    const int depth = CV_MAT_DEPTH(type), cn = CV_MAT_CN(type);
    for (int c = 0; c < cn; ++c) {
        const double v = s.val[c < 4 ? c : 3];
        convertAny(&v, CV_64F, p + c * depthSize(depth), depth, 1);
    }
}
}  // namespace detail

/* 2-D image with shared ownership of its buffer (OpenCV's Mat header
   semantics: copies share data, create() reallocates only when the size or
   type changes).  Buffers carry 64 bytes of zeroed slack past the last
   row, because the reference's bilinear sampler reads one element past the
   row end at x = W - 1. */
class Mat {
public:
    int rows = 0, cols = 0;
    size_t step = 0;
    uchar* data = nullptr;

    Mat() {}
    Mat(int r, int c, int type) { create(r, c, type); }
    Mat(Size s, int type) { create(s.height, s.width, type); }
    Mat(int r, int c, int type, void* ptr, size_t st = 0)
        : rows(r), cols(c), data((uchar*)ptr), type_(type)
    {
        step = st ? st : (size_t)c * elemSize();
    }
    Mat(Size s, int type, void* ptr, size_t st = 0) : Mat(s.height, s.width, type, ptr, st) {}

    void create(int r, int c, int type)
    {
        if (data && r == rows && c == cols && type == type_) return;
        type_ = type;
        rows = r;
        cols = c;
        step = (size_t)c * elemSize();
        const size_t bytes = step * (size_t)r + 64;
        buf_ = std::shared_ptr<uchar>((uchar*)std::calloc(bytes, 1), std::free);
        if (!buf_) throw std::bad_alloc();
        data = buf_.get();
    }
    void create(Size s, int type) { create(s.height, s.width, type); }
    void release() { buf_.reset(); data = nullptr; rows = cols = 0; step = 0; }

    int type() const { return type_; }
    int depth() const { return CV_MAT_DEPTH(type_); }
    int channels() const { return CV_MAT_CN(type_); }
    size_t elemSize() const { return depthSize(depth()) * channels(); }
    size_t elemSize1() const { return depthSize(depth()); }
    Size size() const { return Size(cols, rows); }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    bool isContinuous() const { return step == (size_t)cols * elemSize(); }

    template <class T = uchar> T* ptr(int r) { return (T*)(data + step * (size_t)r); }
    template <class T = uchar> const T* ptr(int r) const { return (const T*)(data + step * (size_t)r); }
    template <class T> T& at(int r, int c) { return ptr<T>(r)[c]; }
    template <class T> const T& at(int r, int c) const { return ptr<T>(r)[c]; }

    Mat& setTo(const Scalar& s, const Mat& mask = Mat())
    {
        for (int r = 0; r < rows; ++r) {
            uchar* p = ptr(r);
            const uchar* m = mask.data ? mask.ptr(r) : nullptr;
            for (int c = 0; c < cols; ++c)
                if (!m || m[c]) detail::setElem(p + c * elemSize(), type_, s);
        }
        return *this;
    }
    void copyTo(Mat& dst) const
    {
        if (dst.data == data) return;
        dst.create(rows, cols, type_);
        for (int r = 0; r < rows; ++r) std::memcpy(dst.ptr(r), ptr(r), (size_t)cols * elemSize());
    }
    void copyTo(Mat& dst, const Mat& mask) const
    {
        dst.create(rows, cols, type_);
        const size_t es = elemSize();
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c)
                if (mask.ptr(r)[c]) std::memcpy(dst.ptr(r) + c * es, ptr(r) + c * es, es);
    }
    Mat clone() const { Mat m; copyTo(m); return m; }
    void convertTo(Mat& dst, int rtype, double alpha = 1, double beta = 0) const
    {
        if (alpha != 1 || beta != 0) throw std::runtime_error("convertTo: scaling is not emulated");
        const int ddepth = rtype < 0 ? depth() : CV_MAT_DEPTH(rtype);
        const Mat src = *this;  /* keeps the source alive if dst aliases it */
        Mat out(rows, cols, CV_MAKETYPE(ddepth, channels()));
        for (int r = 0; r < rows; ++r)
            detail::convertAny(src.ptr(r), depth(), out.ptr(r), ddepth, (size_t)cols * channels());
        dst = out;
    }
    static Mat zeros(int r, int c, int type) { return Mat(r, c, type); }
    static Mat zeros(Size s, int type) { return Mat(s, type); }

private:
    int type_ = 0;
    std::shared_ptr<uchar> buf_;
};

namespace detail {
template <class T> inline void binaryOp(const Mat& a, const Mat& b, Mat& dst, int sign)
{
    CV_Assert(a.size() == b.size() && a.type() == b.type());
    const Mat sa = a, sb = b;  /* dst may alias either operand */
    dst.create(a.rows, a.cols, a.type());
    const size_t n = (size_t)a.cols * a.channels();
    for (int r = 0; r < a.rows; ++r) {
        const T* pa = sa.ptr<T>(r);
        const T* pb = sb.ptr<T>(r);
        T* pd = dst.ptr<T>(r);
        for (size_t i = 0; i < n; ++i) {
            if (std::numeric_limits<T>::is_integer && sizeof(T) < sizeof(int))
                pd[i] = saturate_cast<T>(sign > 0 ? (int)pa[i] + (int)pb[i] : (int)pa[i] - (int)pb[i]);
            else
                pd[i] = (T)(sign > 0 ? pa[i] + pb[i] : pa[i] - pb[i]);
        }
    }
}
inline void arith(const Mat& a, const Mat& b, Mat& dst, int sign)
{
    switch (a.depth()) {
    case CV_8U: binaryOp<uchar>(a, b, dst, sign); break;
    case CV_8S: binaryOp<schar>(a, b, dst, sign); break;
    case CV_16U: binaryOp<ushort>(a, b, dst, sign); break;
    case CV_16S: binaryOp<short>(a, b, dst, sign); break;
    case CV_32S: binaryOp<int>(a, b, dst, sign); break;
    case CV_32F: binaryOp<float>(a, b, dst, sign); break;
    case CV_64F: binaryOp<double>(a, b, dst, sign); break;
    }
}
template <class F> inline Mat bytewise(const Mat& a, const Mat* b, F f)
{
    if (b) CV_Assert(a.size() == b->size() && a.type() == b->type());
    Mat out(a.rows, a.cols, a.type());
    const size_t n = (size_t)a.cols * a.elemSize();
    for (int r = 0; r < a.rows; ++r)
        for (size_t i = 0; i < n; ++i) out.ptr(r)[i] = f(a.ptr(r)[i], b ? b->ptr(r)[i] : (uchar)0);
    return out;
}
}  // namespace detail

inline void add(const Mat& a, const Mat& b, Mat& dst) { detail::arith(a, b, dst, 1); }
inline void subtract(const Mat& a, const Mat& b, Mat& dst) { detail::arith(a, b, dst, -1); }
inline void bitwise_not(const Mat& a, Mat& dst) { dst = detail::bytewise(a, nullptr, [](uchar x, uchar) { return (uchar)~x; }); }
inline Mat operator~(const Mat& a) { return detail::bytewise(a, nullptr, [](uchar x, uchar) { return (uchar)~x; }); }
inline Mat operator&(const Mat& a, const Mat& b) { return detail::bytewise(a, &b, [](uchar x, uchar y) { return (uchar)(x & y); }); }
inline Mat operator|(const Mat& a, const Mat& b) { return detail::bytewise(a, &b, [](uchar x, uchar y) { return (uchar)(x | y); }); }
inline Mat& operator&=(Mat& a, const Mat& b) { a = a & b; return a; }
inline Mat& operator|=(Mat& a, const Mat& b) { a = a | b; return a; }
inline Mat& operator-=(Mat& a, const Mat& b) { subtract(a, b, a); return a; }
inline int countNonZero(const Mat& a)
{
    CV_Assert(a.channels() == 1);
    int c = 0;
    const size_t es = a.elemSize();
    for (int r = 0; r < a.rows; ++r)
        for (int x = 0; x < a.cols; ++x) {
            const uchar* p = a.ptr(r) + x * es;
            bool nz = false;
            for (size_t k = 0; k < es; ++k) nz |= p[k] != 0;
            c += nz;
        }
    return c;
}
inline std::ostream& operator<<(std::ostream& o, const Mat&) { return o << "[Mat]"; }

inline void split(const Mat& m, Mat* out)
{
    const int cn = m.channels();
    const size_t es = m.elemSize1();
    for (int c = 0; c < cn; ++c) {
        out[c].create(m.rows, m.cols, CV_MAKETYPE(m.depth(), 1));
        for (int r = 0; r < m.rows; ++r)
            for (int x = 0; x < m.cols; ++x)
                std::memcpy(out[c].ptr(r) + x * es, m.ptr(r) + (x * cn + c) * es, es);
    }
}

class ParallelLoopBody {
public:
    virtual ~ParallelLoopBody() {}
    virtual void operator()(const Range& range) const = 0;
};

/* Row ranges of one row each, spread over host threads. */
void parallel_for_(const Range& range, const ParallelLoopBody& body, double nstripes = -1.);

}  // namespace cv

#endif
