// Named image buffers, their registry and output selection: the host-side
// buffer surface of the reference's statistics code (class Buffer,
// BufferRegistry and OutputBufferSelection, src/statistics/buffer.h:19-71,
// buffer.cpp:8-63), with the reference's file naming for PFM output and for the
// denoise-only replay (statpath.cpp:506-547).
//
// A Buffer here is planar ([channels][height][width], as the device kernels
// read it) and holds int32, float or double elements; files are always float32,
// as the reference converts every buffer to CV_32F before writing
// (OutputBufferSelection::PrepareOutput, buffer.cpp:41-45).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <filesystem>
#include <functional>
#include <memory>
#include <regex>
#include <string>
#include <vector>

#include "pfm.hpp"

namespace stater {
namespace host {

enum class Elem { I32, F32, F64 };

inline size_t elem_size(Elem e) { return e == Elem::F64 ? 8 : 4; }

struct Buffer {
    std::string name;
    int width = 0, height = 0, channels = 1;
    Elem elem = Elem::F32;
    void *host = nullptr;    // planar host copy (owned through host_owner)
    void *device = nullptr;  // planar device buffer (not owned)
    std::shared_ptr<void> host_owner;
    bool host_dirty = false;  // host copy changed (read from a file) and is due for upload

    size_t elems() const { return (size_t)width * height * channels; }
    size_t bytes() const { return elems() * elem_size(elem); }

    // Host copy as float32 (PrepareOutput's convertTo(CV_32F)).
    std::vector<float> to_float() const {
        std::vector<float> out(elems());
        for (size_t i = 0; i < out.size(); i++) {
            switch (elem) {
                case Elem::I32: out[i] = (float)((const int32_t *)host)[i]; break;
                case Elem::F32: out[i] = ((const float *)host)[i]; break;
                case Elem::F64: out[i] = (float)((const double *)host)[i]; break;
            }
        }
        return out;
    }
    // Host copy from float32 (ReadFile's convertTo(buf.mat.type()): integers
    // rounded to nearest).
    void from_float(const float *v) {
        for (size_t i = 0; i < elems(); i++) {
            switch (elem) {
                case Elem::I32: ((int32_t *)host)[i] = (int32_t)std::lrint(v[i]); break;
                case Elem::F32: ((float *)host)[i] = v[i]; break;
                case Elem::F64: ((double *)host)[i] = (double)v[i]; break;
            }
        }
        host_dirty = true;
    }
};

// Host allocation with a caller-chosen allocator (pinned memory in the Estimator).
using HostAlloc = std::function<std::shared_ptr<void>(size_t)>;

inline std::shared_ptr<void> malloc_host(size_t bytes) {
    void *p = std::calloc(bytes ? bytes : 1, 1);
    if (!p) throw std::bad_alloc();
    return std::shared_ptr<void>(p, [](void *q) { std::free(q); });
}

inline void alloc_host(Buffer &b, const HostAlloc &alloc = malloc_host) {
    if (b.host) return;
    b.host_owner = alloc(b.bytes());
    b.host = b.host_owner.get();
}

// BufferRegistry::Register (buffer.cpp:8-10): every buffer that may be written.
class BufferRegistry {
  public:
    void Register(Buffer &b) { buffers.push_back(&b); }
    std::vector<Buffer *> buffers;
};

// OutputBufferSelection (buffer.cpp:12-63): the registry's buffers whose name
// matches a regex, written as <stem>[-<suffix>]-<name>.<ext>.
class OutputBufferSelection {
  public:
    OutputBufferSelection(const BufferRegistry &reg, const std::string &filename) {
        SetFilename(filename);
        for (Buffer *b : reg.buffers) buffers.push_back(b);
    }
    OutputBufferSelection(const BufferRegistry &reg, const std::regex &regex, const std::string &filename) {
        SetFilename(filename);
        for (Buffer *b : reg.buffers)
            if (std::regex_match(b->name, regex)) buffers.push_back(b);
    }
    std::string GetFilenameStem() const { return filenameStem; }
    std::string FilenameFor(const Buffer &b, const std::string &suffix) const {
        return (suffix.empty() ? filenameStem : filenameStem + "-" + suffix) + "-" + b.name + "." + filenameExtension;
    }
    // Writes every selected buffer's host copy. Only the pfm extension is supported.
    bool Write(const std::string &suffix, std::string *err = nullptr) const {
        if (filenameExtension != "pfm") {
            if (err) *err = "OutputBufferSelection: only .pfm output is supported";
            return false;
        }
        for (const Buffer *b : buffers) {
            if (!b->host) {
                if (err) *err = "OutputBufferSelection: buffer " + b->name + " has no host copy";
                return false;
            }
            const std::vector<float> v = b->to_float();
            if (!write_pfm(FilenameFor(*b, suffix), b->width, b->height, b->channels, v.data(), err)) return false;
        }
        return true;
    }
    std::vector<Buffer *> buffers;

  private:
    void SetFilename(const std::string &filename) {
        const size_t pos = filename.find_last_of('.');
        filenameStem = filename.substr(0, pos);
        filenameExtension = pos == std::string::npos ? "" : filename.substr(pos + 1);
    }
    std::string filenameStem, filenameExtension;
};

// The identifier of a replay file "<stem>-<spp>-<id>.pfm" (statpath.cpp:520-531):
// id = "t<T>-b<j>-<suffix>", where suffix is "film-<name>" for the
// untransformed (t0) set and "<name>" for the transformed (t1) set.
struct BufferFileId {
    int t = -1, b = -1;
    std::string suffix;
};

inline BufferFileId parse_buffer_file_id(const std::string &id) {
    BufferFileId r;
    std::smatch m;
    if (std::regex_search(id, m, std::regex("^t([0-9]+)-"))) r.t = std::stoi(m[1]);
    if (std::regex_search(id, m, std::regex("^t[0-9]+-b([0-9]+)-"))) r.b = std::stoi(m[1]);
    if (std::regex_search(id, m, std::regex("^t[0-9]+-b[0-9]+-(.*)"))) r.suffix = m[1];
    return r;
}

// Files "<prefix>*.pfm" (the cv::glob of statpath.cpp:513-517), sorted, with
// their id (the part between the prefix and ".pfm").
inline std::vector<std::pair<std::string, std::string>> list_replay_files(const std::string &prefix) {
    namespace fs = std::filesystem;
    std::vector<std::pair<std::string, std::string>> out;
    const fs::path pp(prefix);
    const fs::path dir = pp.has_parent_path() ? pp.parent_path() : fs::path(".");
    const std::string base = pp.filename().string();
    std::error_code ec;
    for (const auto &e : fs::directory_iterator(dir, ec)) {
        const std::string fn = e.path().filename().string();
        if (fn.size() > base.size() + 4 && fn.compare(0, base.size(), base) == 0 &&
            fn.compare(fn.size() - 4, 4, ".pfm") == 0)
            out.emplace_back(e.path().string(), fn.substr(base.size(), fn.size() - base.size() - 4));
    }
    std::sort(out.begin(), out.end());
    return out;
}

// Reads a PFM file into a buffer's host copy (StatPathIntegrator::ReadFile).
inline bool read_buffer(const std::string &path, Buffer &b, std::string *err = nullptr,
                        const HostAlloc &alloc = malloc_host) {
    PfmImage img;
    if (!read_pfm(path, img, err)) return false;
    if (img.width != b.width || img.height != b.height || img.channels != b.channels) {
        if (err) *err = "read_buffer: " + path + " does not match buffer " + b.name;
        return false;
    }
    alloc_host(b, alloc);
    b.from_float(img.planar.data());
    return true;
}

}  // namespace host
}  // namespace stater
