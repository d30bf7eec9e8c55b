// CPU checks of the host-side buffer surface (stater_gb300/host/buffer.hpp,
// pfm.hpp): PFM round trips, byte order, the reference's output file naming
// (buffer.cpp:48-63), replay file ids (statpath.cpp:520-531) and the integer
// rounding of ReadFile's convertTo. Prints "OK" and exits 0 on success.
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <string>

#include "buffer.hpp"

using namespace stater::host;

#define REQUIRE(c)                                                          \
    do {                                                                    \
        if (!(c)) {                                                         \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__); \
            return 1;                                                       \
        }                                                                   \
    } while (0)

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    std::string err;

    // 3-channel round trip, rows stored bottom to top
    const int W = 5, H = 3;
    std::vector<float> img(3 * W * H);
    for (size_t i = 0; i < img.size(); i++) img[i] = 0.25f * (float)i - 3.0f;
    REQUIRE(write_pfm(dir + "/rgb.pfm", W, H, 3, img.data(), &err));
    PfmImage back;
    REQUIRE(read_pfm(dir + "/rgb.pfm", back, &err));
    REQUIRE(back.width == W && back.height == H && back.channels == 3);
    REQUIRE(back.planar == img);
    {
        std::FILE *f = std::fopen((dir + "/rgb.pfm").c_str(), "rb");
        char head[32] = {0};
        REQUIRE(std::fread(head, 1, 14, f) == 14);
        std::fclose(f);
        REQUIRE(std::string(head, 12) == "PF\n5 3\n-1.0\n");
    }

    // 1-channel, big-endian file written by hand
    {
        const std::string p = dir + "/be.pfm";
        std::FILE *f = std::fopen(p.c_str(), "wb");
        std::fprintf(f, "Pf\n2 1\n1.0\n");
        const unsigned char v[8] = {0x3f, 0x80, 0x00, 0x00, 0xc0, 0x00, 0x00, 0x00};  // 1.0, -2.0
        std::fwrite(v, 1, 8, f);
        std::fclose(f);
        PfmImage g;
        REQUIRE(read_pfm(p, g, &err));
        REQUIRE(g.channels == 1 && g.planar.size() == 2 && g.planar[0] == 1.0f && g.planar[1] == -2.0f);
    }
    // truncated file and bad header are errors
    {
        const std::string p = dir + "/bad.pfm";
        std::FILE *f = std::fopen(p.c_str(), "wb");
        std::fprintf(f, "PF\n4 4\n-1\n");
        std::fwrite(img.data(), 4, 3, f);
        std::fclose(f);
        PfmImage g;
        REQUIRE(!read_pfm(p, g, &err));
        f = std::fopen(p.c_str(), "wb");
        std::fprintf(f, "P6\n4 4\n255\n");
        std::fclose(f);
        REQUIRE(!read_pfm(p, g, &err));
    }

    // registry, regex selection and file names
    Buffer a, b, n;
    a.name = "t0-b0-film-mean"; a.width = W; a.height = H; a.channels = 3;
    b.name = "t0-b1-varD";      b.width = W; b.height = H; b.channels = 3;
    n.name = "t0-b0-film-n";    n.width = W; n.height = H; n.channels = 1; n.elem = Elem::I32;
    alloc_host(a); alloc_host(b); alloc_host(n);
    for (int i = 0; i < 3 * W * H; i++) ((float *)a.host)[i] = (float)i;
    for (int i = 0; i < W * H; i++) ((int32_t *)n.host)[i] = 1000 + i;
    BufferRegistry reg;
    reg.Register(a); reg.Register(b); reg.Register(n);
    OutputBufferSelection sel(reg, std::regex(".*film.*"), dir + "/scene.pfm");
    REQUIRE(sel.buffers.size() == 2);
    REQUIRE(sel.GetFilenameStem() == dir + "/scene");
    REQUIRE(sel.FilenameFor(a, "64") == dir + "/scene-64-t0-b0-film-mean.pfm");
    REQUIRE(sel.FilenameFor(a, "") == dir + "/scene-t0-b0-film-mean.pfm");
    REQUIRE(sel.Write("64", &err));
    REQUIRE(std::filesystem::exists(dir + "/scene-64-t0-b0-film-n.pfm"));
    REQUIRE(!std::filesystem::exists(dir + "/scene-64-t0-b1-varD.pfm"));
    OutputBufferSelection bad(reg, dir + "/scene.exr");
    REQUIRE(!bad.Write("64", &err));

    // replay ids: "film-<name>" is the untransformed set, "<name>" the transformed one
    BufferFileId id = parse_buffer_file_id("t0-b3-film-m2");
    REQUIRE(id.t == 0 && id.b == 3 && id.suffix == "film-m2");
    id = parse_buffer_file_id("t12-b0-varCD");
    REQUIRE(id.t == 12 && id.b == 0 && id.suffix == "varCD");
    id = parse_buffer_file_id("film");
    REQUIRE(id.t == -1 && id.b == -1 && id.suffix.empty());
    auto files = list_replay_files(dir + "/scene-64-");
    REQUIRE(files.size() == 2);
    REQUIRE(files[0].second == "t0-b0-film-mean" && files[1].second == "t0-b0-film-n");

    // read back: floats exact, integers through float and rounded
    Buffer a2 = a, n2 = n;
    a2.host = nullptr; a2.host_owner.reset();
    n2.host = nullptr; n2.host_owner.reset();
    REQUIRE(read_buffer(files[0].first, a2, &err) && a2.host_dirty);
    REQUIRE(read_buffer(files[1].first, n2, &err));
    for (int i = 0; i < 3 * W * H; i++) REQUIRE(((float *)a2.host)[i] == (float)i);
    for (int i = 0; i < W * H; i++) REQUIRE(((int32_t *)n2.host)[i] == 1000 + i);
    Buffer wrong = a2;
    wrong.channels = 1;
    REQUIRE(!read_buffer(files[0].first, wrong, &err));
    std::printf("OK\n");
    return 0;
}
