// Stand-in for src/statistics/buffer.h: only the names that estimator.h's
// Estimator declaration mentions. StatTile does not use any of it.
#pragma once
#include <string>
#include <vector>
#include "statistics/statpbrt.h"
namespace pbrt {
class Buffer {
  public:
    Buffer() {}
    Buffer(const std::string &, Mat) {}
    Mat mat;
    GpuMat gpuMat;
};
class BufferRegistry {
  public:
    void Register(const Buffer &) {}
};
}  // namespace pbrt
