// loaders.cpp -- OBJ and STL loading the way the reference's loaders see the files.
//
// The reference calls two crates whose sources are not in its tree: tobj 3.2.2
// (src/inputs.rs:108-113, load_obj with GPU_LOAD_OPTIONS: single_index, triangulate,
// ignore points and lines) and stl_io 0.4.2 (src/inputs.rs:116-121, read_stl).  This file
// restates their published behaviour for what the reference uses -- positions, face and
// material structure, diffuse colours, vertex colours -- and then the reference's own
// conversion to SimpleMesh (src/geometry.rs:83-189).  Numbers are parsed with strtof
// (correctly rounded, like Rust's f32::from_str).
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>

#include "sloth_host.hpp"

namespace sloth_host {

namespace {

std::vector<std::string> split_ws(const std::string &line)
{
    std::vector<std::string> out;
    std::istringstream is(line);
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
}

bool parse_f32(const std::string &s, float *v)
{
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    const float f = std::strtof(s.c_str(), &end);
    if (end != s.c_str() + s.size()) return false;
    *v = f;
    return true;
}

// Rust `(f * 255.0) as u8` on an f32: the product rounded to f32, then a saturating
// truncation (NaN -> 0).
uint8_t unit_to_u8(float f)
{
    const volatile float p = f * 255.0f;
    const float q = p;
    if (!(q > 0.0f)) return 0;
    if (q >= 255.0f) return 255;
    return (uint8_t)q;
}

// Triangle::aabb (src/geometry.rs:37-42) folded into the mesh box (src/geometry.rs:128-133),
// with Rust's NaN-ignoring f32::min/max.
void add_triangle(SimpleMesh &m, const float v[9], const uint8_t c[3])
{
    for (int k = 0; k < 3; ++k) {
        m.x.push_back(v[3 * k]);
        m.y.push_back(v[3 * k + 1]);
        m.z.push_back(v[3 * k + 2]);
    }
    m.rgb.insert(m.rgb.end(), c, c + 3);
    for (int a = 0; a < 3; ++a) {
        const float mn = std::fmin(v[a], std::fmin(v[3 + a], v[6 + a]));
        const float mx = std::fmax(v[a], std::fmax(v[3 + a], v[6 + a]));
        m.bbox_min[a] = std::fmin(mn, m.bbox_min[a]);
        m.bbox_max[a] = std::fmax(mx, m.bbox_max[a]);
    }
}

// The rest of a line after its first word, trimmed (material names may hold spaces).
std::string rest_of_line(const std::string &line, const std::string &tag)
{
    size_t a = line.find(tag);
    a = a == std::string::npos ? line.size() : a + tag.size();
    const size_t b = line.find_first_not_of(" \t\r", a);
    if (b == std::string::npos) return std::string();
    const size_t e = line.find_last_not_of(" \t\r");
    return line.substr(b, e - b + 1);
}

struct Material {
    std::string name;
    float kd[3] = {0, 0, 0};
};

// The diffuse colours of an MTL file, materials in file order.
bool load_mtl(const std::string &path, std::vector<Material> &mats)
{
    std::ifstream in(path);
    if (!in) return false;
    std::string line;
    while (std::getline(in, line)) {
        const auto t = split_ws(line);
        if (t.empty() || t[0][0] == '#') continue;
        if (t[0] == "newmtl") {
            Material m;
            m.name = rest_of_line(line, "newmtl");
            mats.push_back(m);
        } else if (t[0] == "Kd" && !mats.empty() && t.size() >= 4) {
            for (int k = 0; k < 3; ++k)
                if (!parse_f32(t[1 + k], &mats.back().kd[k])) return false;
        }
    }
    return true;
}

std::string dir_of(const std::string &path)
{
    const size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

}  // namespace

std::vector<SimpleMesh> load_obj(const std::string &path)
{
    std::ifstream in(path);
    if (!in) throw LoadError("tobj couldnt load/parse OBJ. Unable to open file");
    std::vector<float> pos, vcol;
    std::vector<Material> mats;
    bool mtl_failed = false;
    struct Model {
        std::vector<uint32_t> corners;   // 3 position indices per triangle
        int mat;                          // -1: none
    };
    std::vector<Model> models;
    std::vector<uint32_t> faces;
    int mat = -1;
    auto push_model = [&]() {
        if (!faces.empty()) models.push_back(Model{faces, mat});
        faces.clear();
    };
    std::string line;
    while (std::getline(in, line)) {
        const auto t = split_ws(line);
        if (t.empty() || t[0][0] == '#') continue;
        const std::string &tag = t[0];
        if (tag == "v") {
            float v[6];
            const size_t n = t.size() - 1;
            if (n < 3) throw LoadError("tobj couldnt load/parse OBJ. PositionParseError");
            for (size_t k = 0; k < 3; ++k)
                if (!parse_f32(t[1 + k], &v[k])) throw LoadError("tobj couldnt load/parse OBJ. PositionParseError");
            pos.insert(pos.end(), v, v + 3);
            if (n >= 6) {
                for (size_t k = 3; k < 6; ++k)
                    if (!parse_f32(t[1 + k], &v[k])) throw LoadError("tobj couldnt load/parse OBJ. PositionParseError");
                vcol.insert(vcol.end(), v + 3, v + 6);
            }
        } else if (tag == "f") {
            std::vector<uint32_t> ids;
            const long nv = (long)(pos.size() / 3);
            for (size_t k = 1; k < t.size(); ++k) {
                const std::string idx = t[k].substr(0, t[k].find('/'));
                char *end = nullptr;
                const long i = std::strtol(idx.c_str(), &end, 10);
                if (idx.empty() || *end || i == 0) throw LoadError("tobj couldnt load/parse OBJ. FaceParseError");
                const long j = i > 0 ? i - 1 : nv + i;
                if (j < 0 || j >= nv) throw LoadError("tobj couldnt load/parse OBJ. FaceVertexOutOfBounds");
                ids.push_back((uint32_t)j);
            }
            if (ids.size() < 3) continue;   // points and lines are ignored
            for (size_t k = 1; k + 1 < ids.size(); ++k) {
                faces.push_back(ids[0]);
                faces.push_back(ids[k]);
                faces.push_back(ids[k + 1]);
            }
        } else if (tag == "o" || tag == "g") {
            push_model();
        } else if (tag == "usemtl") {
            const std::string name = rest_of_line(line, "usemtl");
            if (name.empty()) throw LoadError("tobj couldnt load/parse OBJ. MaterialParseError");
            int found = -1;
            for (size_t k = 0; k < mats.size() && found < 0; ++k)
                if (mats[k].name == name) found = (int)k;
            // a new model starts when a known material differs from the current one
            if (found >= 0 && found != mat) push_model();
            mat = found;
        } else if (tag == "mtllib") {
            if (t.size() >= 2 && !load_mtl(dir_of(path) + t[1], mats)) mtl_failed = true;
        }
    }
    push_model();
    if (mtl_failed) throw LoadError("Expected to have materials.");
    std::vector<SimpleMesh> out;
    const bool colours = !vcol.empty();
    for (const Model &md : models) {
        SimpleMesh m;
        for (size_t t3 = 0; t3 < md.corners.size(); t3 += 3) {
            float v[9];
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) v[3 * k + a] = pos[3 * (size_t)md.corners[t3 + k] + a];
            uint8_t c[3] = {1, 1, 1};
            if (!mats.empty()) {
                if (md.mat < 0) throw LoadError("called `Option::unwrap()` on a `None` value (no material)");
                for (int a = 0; a < 3; ++a) c[a] = unit_to_u8(mats[(size_t)md.mat].kd[a]);
                if (colours) {
                    const size_t vi = md.corners[t3];
                    if (3 * vi + 2 >= vcol.size()) throw LoadError("vertex colour index out of range");
                    for (int a = 0; a < 3; ++a) c[a] = unit_to_u8(vcol[3 * vi + a]);
                }
            }
            add_triangle(m, v, c);
        }
        out.push_back(std::move(m));
    }
    return out;
}

SimpleMesh load_stl(const std::string &path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw LoadError("STL load failed. Unable to open file");
    std::string data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    SimpleMesh m;
    const float mx = std::numeric_limits<float>::max();
    m.bbox_min[0] = m.bbox_min[1] = m.bbox_min[2] = mx;
    m.bbox_max[0] = m.bbox_max[1] = m.bbox_max[2] = -mx;
    const uint8_t yellow[3] = {255, 255, 0};
    if (data.compare(0, 6, "solid ") == 0) {
        std::istringstream is(data);
        std::string line;
        float v[9];
        int nv = 0;
        while (std::getline(is, line)) {
            const auto t = split_ws(line);
            if (t.empty() || t[0] != "vertex") continue;
            if (t.size() < 4) throw LoadError("stl_io couldnt parse STL. bad vertex");
            for (int a = 0; a < 3; ++a)
                if (!parse_f32(t[1 + a], &v[3 * nv + a])) throw LoadError("stl_io couldnt parse STL. bad vertex");
            if (++nv == 3) {
                add_triangle(m, v, yellow);
                nv = 0;
            }
        }
        if (nv) throw LoadError("stl_io couldnt parse STL. incomplete facet");
    } else {
        if (data.size() < 84) throw LoadError("stl_io couldnt parse STL. short header");
        uint32_t n;
        std::memcpy(&n, data.data() + 80, 4);
        if (data.size() < 84 + 50 * (size_t)n) throw LoadError("stl_io couldnt parse STL. short file");
        for (uint32_t i = 0; i < n; ++i) {
            float v[9];
            std::memcpy(v, data.data() + 84 + 50 * (size_t)i + 12, 36);
            add_triangle(m, v, yellow);
        }
    }
    return m;
}

std::vector<SimpleMesh> match_meshes(const std::string &files)
{
    std::vector<SimpleMesh> queue;
    size_t a = 0;
    for (;;) {
        const size_t b = files.find(' ', a);
        const std::string slice = files.substr(a, b == std::string::npos ? std::string::npos : b - a);
        auto error = [&](const std::string &s, const std::string &e) {
            return LoadError("filename: [" + slice + "] couldn't load, " + s + ". " + e);
        };
        const size_t dot = slice.find_last_of('.');
        const size_t slash = slice.find_last_of('/');
        if (dot == std::string::npos || (slash != std::string::npos && dot < slash) || dot == 0 ||
            (slash != std::string::npos && dot == slash + 1))
            throw error("couldn't determine filename extension", "");
        std::string ext = slice.substr(dot + 1);
        std::transform(ext.begin(), ext.end(), ext.begin(), [](unsigned char ch) { return (char)std::tolower(ch); });
        try {
            if (ext == "obj") {
                auto ms = load_obj(slice);
                for (auto &m : ms) queue.push_back(std::move(m));
            } else if (ext == "stl") {
                queue.push_back(load_stl(slice));
            } else {
                throw error("unknown filename extension", "");
            }
        } catch (const LoadError &e) {
            const std::string msg = e.what();
            if (msg.rfind("filename: [", 0) == 0 || msg == "Expected to have materials.") throw;
            const size_t sep = msg.find(". ");
            throw error(msg.substr(0, sep), sep == std::string::npos ? "" : msg.substr(sep + 2));
        }
        if (b == std::string::npos) break;
        a = b + 1;
    }
    return queue;
}

}  // namespace sloth_host
