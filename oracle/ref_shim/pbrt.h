// Stand-in for pbrt's core header, just large enough for the reference's
// src/statistics/estimator.h (StatTile / Tile) to compile without pbrt-v3.
// Provides Float (float, or double with -DPBRT_FLOAT_AS_DOUBLE as in
// src/core/pbrt.h:169-173), Point2i/Point2f, Vector2f and Bounds2i with the
// members the header touches (x, y, pMin, pMax, Area()).
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <algorithm>
#include <cmath>

namespace pbrt {
#ifdef PBRT_FLOAT_AS_DOUBLE
typedef double Float;
#else
typedef float Float;
#endif

template <typename T> struct Point2 {
    T x{}, y{};
    Point2() {}
    Point2(T x, T y) : x(x), y(y) {}
};
typedef Point2<int> Point2i;
typedef Point2<Float> Point2f;

template <typename T> struct Vector2 {
    T x{}, y{};
    Vector2() {}
    Vector2(T x, T y) : x(x), y(y) {}
};
typedef Vector2<Float> Vector2f;

struct Bounds2i {
    Point2i pMin, pMax;
    Bounds2i() {}
    Bounds2i(Point2i a, Point2i b) : pMin(a), pMax(b) {}
    int Area() const { return (pMax.x - pMin.x) * (pMax.y - pMin.y); }
};
}  // namespace pbrt
