// Stand-in for src/statistics/statpbrt.h. Provides the macro defaults of the
// reference (statpbrt.h:11-29) and a minimal element-wise cv::Vec<T,3> whose
// operators follow OpenCV's Vec semantics for floating types (each element is
// computed independently with one IEEE operation: a[i]-b[i], a[i]+b[i],
// a[i]*alpha). Element-wise Vec*Vec, Vec/uint64 and sqrt(Vec) come from the
// reference header itself (estimator.h:23-40). The OpenCV matrix, GPU matrix
// and stream types are empty placeholders: only Estimator's inline constructor
// names them and it is never instantiated by the harness.
#pragma once
#ifndef DEBUG
#define DEBUG 0
#endif
#ifndef STATMC
#define STATMC 0
#endif
#ifndef DISABLE_DENOISE_VARS
#define DISABLE_DENOISE_VARS 0
#endif
#ifndef FULL_MULTI_TRANSFORM
#define FULL_MULTI_TRANSFORM 0
#endif
#ifndef FILM_MULTI_TRANSFORM_MODE
#define FILM_MULTI_TRANSFORM_MODE 2
#endif
#define STRINGIFY(x) #x
#define TOSTRING(x) STRINGIFY(x)
#define SHOW_MACRO(m)

#include <string>
#include <vector>
#include <cstdint>
#include <algorithm>
#include <iterator>
#include <unordered_set>
#include "pbrt.h"

typedef unsigned char uchar;

namespace cv {
template <typename T, int cn> struct Vec {
    T val[cn];
    Vec() { for (int i = 0; i < cn; i++) val[i] = T(0); }
    Vec(T a, T b, T c) { val[0] = a; val[1] = b; val[2] = c; }
    explicit Vec(const T *v) { for (int i = 0; i < cn; i++) val[i] = v[i]; }
    T &operator[](int i) { return val[i]; }
    const T &operator[](int i) const { return val[i]; }
};
template <typename T, int cn> inline Vec<T, cn> operator+(const Vec<T, cn> &a, const Vec<T, cn> &b) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = a.val[i] + b.val[i]; return r;
}
template <typename T, int cn> inline Vec<T, cn> operator-(const Vec<T, cn> &a, const Vec<T, cn> &b) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = a.val[i] - b.val[i]; return r;
}
template <typename T, int cn> inline Vec<T, cn> &operator+=(Vec<T, cn> &a, const Vec<T, cn> &b) {
    for (int i = 0; i < cn; i++) a.val[i] = a.val[i] + b.val[i]; return a;
}
template <typename T, int cn> inline Vec<T, cn> operator*(const Vec<T, cn> &a, float alpha) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = (T)(a.val[i] * alpha); return r;
}
template <typename T, int cn> inline Vec<T, cn> operator*(float alpha, const Vec<T, cn> &a) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = (T)(a.val[i] * alpha); return r;
}
template <typename T, int cn> inline Vec<T, cn> operator*(const Vec<T, cn> &a, double alpha) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = (T)(a.val[i] * alpha); return r;
}
template <typename T, int cn> inline Vec<T, cn> operator*(double alpha, const Vec<T, cn> &a) {
    Vec<T, cn> r; for (int i = 0; i < cn; i++) r.val[i] = (T)(a.val[i] * alpha); return r;
}
typedef Vec<float, 3> Vec3f;
struct Mat {
    int rows = 0, cols = 0;
    Mat() {}
    Mat(int r, int c, int) : rows(r), cols(c) {}
    template <typename T> Mat(const std::vector<T> &) {}
    static void setDefaultAllocator(void *) {}
};
template <typename T> struct Mat_ : Mat { Mat_() {} Mat_(int r, int c) { rows = r; cols = c; } };
typedef Mat_<float> Mat1f;
typedef Mat_<int> Mat1i;
typedef Mat_<Vec3f> Mat3f;
namespace cuda {
struct GpuMat {};
struct Stream {};
struct HostMem {
    enum AllocType { PAGE_LOCKED = 1 };
    static void *getAllocator(AllocType) { return nullptr; }
};
namespace stat_denoiser {
inline void setup() {}
}  // namespace stat_denoiser
}  // namespace cuda
}  // namespace cv

namespace pbrt {
using cv::Vec3f;
using cv::Mat;
using cv::Mat_;
using cv::Mat1f;
using cv::Mat1i;
using cv::Mat3f;
using cv::cuda::GpuMat;
using Vec3 = cv::Vec<Float, 3>;
using Vec4 = cv::Vec<Float, 4>;
using Mat1 = Mat_<Float>;
using Mat3 = Mat_<Vec3>;
class Estimator;
}  // namespace pbrt
