// Portable float map (PFM) files for statistics buffers: the on-disk format the
// reference writes every buffer in (OutputBufferSelection::Write through
// cv::imwrite, src/statistics/buffer.cpp:48-63) and reads back for denoise-only
// runs (StatPathIntegrator::ReadFile, src/statistics/statpath.cpp:479-484).
//
// Format: "PF" (3 channels, RGB) or "Pf" (1 channel), then width and height,
// then a scale whose sign gives the byte order (negative = little-endian), each
// followed by one whitespace character; then float32 pixels, channels
// interleaved, rows bottom to top. In memory the images here are planar
// [channels][height][width] with row 0 at the top, as the device buffers are.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace stater {
namespace host {

struct PfmImage {
    int width = 0, height = 0, channels = 0;
    std::vector<float> planar;  // [channels][height][width], row 0 = top
};

namespace detail {
inline bool little_endian_host() {
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}
inline uint32_t bswap32(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xFF00u) | ((v << 8) & 0xFF0000u) | (v << 24);
}
inline bool fail(std::string *err, const std::string &msg) {
    if (err) *err = msg;
    return false;
}
// Reads one whitespace-delimited token; consumes exactly one whitespace after it.
inline bool token(std::FILE *f, std::string &out) {
    out.clear();
    int c;
    while ((c = std::fgetc(f)) != EOF && (c == ' ' || c == '\n' || c == '\r' || c == '\t')) {
    }
    while (c != EOF && !(c == ' ' || c == '\n' || c == '\r' || c == '\t')) {
        out.push_back((char)c);
        c = std::fgetc(f);
    }
    return !out.empty();
}
}  // namespace detail

// Writes a planar float image of 1 or 3 channels.
inline bool write_pfm(const std::string &path, int width, int height, int channels, const float *planar,
                      std::string *err = nullptr) {
    if (width <= 0 || height <= 0 || (channels != 1 && channels != 3) || !planar)
        return detail::fail(err, "write_pfm: bad image");
    std::FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return detail::fail(err, "write_pfm: cannot open " + path);
    const bool le = detail::little_endian_host();
    std::fprintf(f, "%s\n%d %d\n%s\n", channels == 3 ? "PF" : "Pf", width, height, le ? "-1.0" : "1.0");
    const size_t plane = (size_t)width * height;
    std::vector<float> row((size_t)width * channels);
    bool ok = true;
    for (int y = height - 1; y >= 0 && ok; y--) {
        for (int x = 0; x < width; x++)
            for (int c = 0; c < channels; c++) row[(size_t)x * channels + c] = planar[c * plane + (size_t)y * width + x];
        ok = std::fwrite(row.data(), sizeof(float), row.size(), f) == row.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? true : detail::fail(err, "write_pfm: write failed for " + path);
}

inline bool read_pfm(const std::string &path, PfmImage &img, std::string *err = nullptr) {
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return detail::fail(err, "read_pfm: cannot open " + path);
    std::string magic, ws, hs, ss;
    const bool head = detail::token(f, magic) && detail::token(f, ws) && detail::token(f, hs) && detail::token(f, ss);
    int channels = magic == "PF" ? 3 : magic == "Pf" ? 1 : 0;
    char *end = nullptr;
    const long w = head ? std::strtol(ws.c_str(), &end, 10) : 0;
    const long h = head ? std::strtol(hs.c_str(), &end, 10) : 0;
    const double scale = head ? std::strtod(ss.c_str(), &end) : 0.0;
    if (!head || channels == 0 || w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16) || scale == 0.0 ||
        !std::isfinite(scale)) {
        std::fclose(f);
        return detail::fail(err, "read_pfm: bad header in " + path);
    }
    const bool file_le = scale < 0.0;
    const bool swap = file_le != detail::little_endian_host();
    img.width = (int)w;
    img.height = (int)h;
    img.channels = channels;
    const size_t plane = (size_t)w * h;
    img.planar.assign(plane * channels, 0.f);
    std::vector<uint32_t> row((size_t)w * channels);
    for (long y = h - 1; y >= 0; y--) {
        if (std::fread(row.data(), sizeof(uint32_t), row.size(), f) != row.size()) {
            std::fclose(f);
            return detail::fail(err, "read_pfm: truncated data in " + path);
        }
        for (long x = 0; x < w; x++)
            for (int c = 0; c < channels; c++) {
                uint32_t v = row[(size_t)x * channels + c];
                if (swap) v = detail::bswap32(v);
                float fv;
                std::memcpy(&fv, &v, 4);
                img.planar[c * plane + (size_t)y * w + x] = fv;
            }
    }
    std::fclose(f);
    return true;
}

}  // namespace host
}  // namespace stater
