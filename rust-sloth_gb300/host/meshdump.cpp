// meshdump.cpp -- writes the meshes the host loaders read from one `sloth` file argument
// as binary on stdout (for the loader tests; no GPU):
//   u32 nmesh; per mesh: u32 ntri, f32 x[3*ntri], f32 y[3*ntri], f32 z[3*ntri],
//   u8 rgb[3*ntri], f32 bbox_min[3], f32 bbox_max[3].
// On a load error: the error text on stderr, exit code 1.
#include <cstdio>

#include "sloth_host.hpp"

int main(int argc, char **argv)
{
    if (argc != 2) {
        std::fprintf(stderr, "usage: sloth_meshdump \"<file> [file ...]\"\n");
        return 2;
    }
    try {
        const auto meshes = sloth_host::match_meshes(argv[1]);
        const uint32_t n = (uint32_t)meshes.size();
        std::fwrite(&n, 4, 1, stdout);
        for (const auto &m : meshes) {
            const uint32_t t = (uint32_t)m.triangles();
            std::fwrite(&t, 4, 1, stdout);
            std::fwrite(m.x.data(), 4, m.x.size(), stdout);
            std::fwrite(m.y.data(), 4, m.y.size(), stdout);
            std::fwrite(m.z.data(), 4, m.z.size(), stdout);
            std::fwrite(m.rgb.data(), 1, m.rgb.size(), stdout);
            std::fwrite(m.bbox_min, 4, 3, stdout);
            std::fwrite(m.bbox_max, 4, 3, stdout);
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
