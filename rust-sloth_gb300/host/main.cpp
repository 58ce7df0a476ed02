// main.cpp -- the `sloth` command for the image path of the reference's main
// (src/main.rs:27-111, arguments src/inputs.rs:9-175), drawing through the GB300 library:
//
//   sloth [-b] [-x a] [-y b] [-z c] "<file> [file ...]" image -w W [-h H] [-x a] [-y b] [-z c] [-j N]
//
// The first positional argument is split on spaces (match_meshes); -b (no colour) is read
// from the top-level options and -x/-y/-z from the image subcommand's, as the reference
// reads them.  Output on stdout is byte-for-byte Context::flush's, and with -j N the JS
// export wrapper (let frames = [ `...`, ... `];) around N turntable frames.  The
// interactive terminal mode (no `image` subcommand) is not part of this build.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sloth_host.hpp"

using namespace sloth_host;

namespace {

constexpr float kPi = 3.14159265358979323846f;

struct Args {
    std::string files;
    bool have_files = false;
    bool image = false;
    bool no_color = false;                       // top-level -b
    const char *rot[3] = {nullptr, nullptr, nullptr};   // -x, -y, -z of the active level
    const char *width = nullptr, *height = nullptr, *frames = nullptr;
};

[[noreturn]] void usage_error(const std::string &msg)
{
    std::fprintf(stderr, "error: %s\n", msg.c_str());
    std::exit(2);
}

Args parse(int argc, char **argv)
{
    Args a;
    const char *top_rot[3] = {nullptr, nullptr, nullptr};
    const char *sub_rot[3] = {nullptr, nullptr, nullptr};
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        auto value = [&](const char *name) -> const char * {
            if (i + 1 >= argc) usage_error(std::string("missing value for ") + name);
            return argv[++i];
        };
        const char **rot = a.image ? sub_rot : top_rot;
        if (s == "-b") {
            if (!a.image) a.no_color = true;
        } else if (s == "-x" || s == "--yaw") {
            rot[0] = value("-x");
        } else if (s == "-y" || s == "--pitch") {
            rot[1] = value("-y");
        } else if (s == "-z" || s == "--roll") {
            rot[2] = value("-z");
        } else if (a.image && s == "-w") {
            a.width = value("-w");
        } else if (a.image && s == "-h") {
            a.height = value("-h");
        } else if (a.image && (s == "-j" || s == "--webify")) {
            a.frames = value("-j");
        } else if (!a.image && s == "image") {
            a.image = true;
        } else if (!s.empty() && s[0] == '-') {
            usage_error("unknown option " + s);
        } else if (!a.image) {
            if (!a.have_files) a.files = s;   // value_of: the first value only
            a.have_files = true;
        } else {
            usage_error("unexpected argument " + s);
        }
    }
    if (!a.have_files) usage_error("the input filename(s) are required");
    for (int k = 0; k < 3; ++k) a.rot[k] = a.image ? sub_rot[k] : top_rot[k];
    if (a.image && !a.width) usage_error("image needs -w");
    return a;
}

// Rust's str::parse::<f32> / ::<usize> / ::<i32>, reporting failures like `?` does.
float parse_f32(const char *s)
{
    char *end = nullptr;
    const float v = std::strtof(s, &end);
    if (!*s || *end) throw std::runtime_error("ParseFloatError { kind: Invalid }");
    return v;
}

long long parse_int(const char *s, bool is_unsigned)
{
    char *end = nullptr;
    if (!*s || (is_unsigned && s[0] == '-')) throw std::runtime_error("ParseIntError { kind: InvalidDigit }");
    const long long v = std::strtoll(s, &end, 10);
    if (*end) throw std::runtime_error("ParseIntError { kind: InvalidDigit }");
    return v;
}

}  // namespace

int main(int argc, char **argv)
{
    const Args args = parse(argc, argv);
    if (!args.image) {
        std::fprintf(stderr, "error: the interactive terminal mode is not part of this build; use `image`\n");
        return 2;
    }
    try {
        const std::vector<SimpleMesh> queue = match_meshes(args.files);
        // match_turntable: (yaw -> roll slot, pitch + pi, roll, speed 1.0)
        float turntable[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        for (int k = 0; k < 3; ++k)
            if (args.rot[k]) turntable[k] = parse_f32(args.rot[k]);
        turntable[1] += kPi;
        Context context(true);
        context.width = (size_t)parse_int(args.width, true);
        context.height = args.height ? (size_t)parse_int(args.height, true) : context.width;
        const bool webify = args.frames != nullptr;
        long long todo = 0, count = 0;
        if (webify) {
            todo = parse_int(args.frames, false);
            std::fputs("let frames = [\n", stdout);
            turntable[3] = (2.0f * kPi) * (1.0f / (float)todo);
        }
        for (;;) {
            float rot[16];
            sloth_euler_rotation(turntable[0], turntable[1], turntable[2], rot);
            context.update(queue);
            context.clear();
            for (const SimpleMesh &m : queue) context.draw_mesh(m, rot);
            if (webify) std::fputs("`\n", stdout);
            context.flush(!args.no_color, webify, stdout);
            std::fflush(stdout);
            if (!webify) break;   // an image without -j is one frame
            turntable[1] += turntable[3];
            if (turntable[1] > 9.42477f || todo - 1 == count) {
                std::fputs("`];\n", stdout);
                break;
            }
            std::fputs("`,\n", stdout);
            ++count;
        }
        std::fflush(stdout);
    } catch (const LoadError &e) {
        if (std::strcmp(e.what(), "Expected to have materials.") == 0) {
            std::fprintf(stderr, "thread 'main' panicked at 'Expected to have materials.'\n");
            return 101;
        }
        std::fprintf(stderr, "Error: \"%s\"\n", e.what());
        return 1;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "Error: %s\n", e.what());
        return 1;
    }
    return 0;
}
