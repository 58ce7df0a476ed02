// sloth_host.hpp -- C++ host side of the GB300 rasterizer, mirroring the reference's Rust
// types and calls for the draw path (the reference's toolchain, cargo, is not available, so
// this is the layer a Rust FFI crate would be):
//   SimpleMesh                     src/geometry.rs:78-81 (+ loaders src/geometry.rs:83-189,
//                                  src/inputs.rs:95-129)
//   Context::blank/clear/update/flush, draw_mesh
//                                  src/context.rs:21-141, src/rasterizer.rs:39-46
// Everything that touches pixels goes through the C ABI of include/sloth_gpu.h.
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "sloth_gpu.h"

namespace sloth_host {

// A list of triangles with one face colour each (the reference's Vec<Triangle>), stored as
// an unindexed soup: triangle t is vertices 3t, 3t+1, 3t+2 of x, y, z.
struct SimpleMesh {
    std::vector<float> x, y, z;
    std::vector<uint8_t> rgb;    // 3 per triangle
    float bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0};
    size_t triangles() const { return rgb.size() / 3; }
};

// Loader failures, with the reference's message text.
struct LoadError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// tobj::load_obj(path, &GPU_LOAD_OPTIONS) + to_simple_mesh_with_materials: one mesh per
// model (object, group or material change), polygons fan-triangulated, colour = material
// diffuse * 255 as u8, replaced by the first corner's vertex colour when the file has
// vertex colours, (1,1,1) without materials; bounding box grown from the origin.
std::vector<SimpleMesh> load_obj(const std::string &path);

// stl_io::read_stl + to_simple_mesh: ASCII when the file starts with "solid ", binary
// otherwise; facets in file order, colour (255,255,0), bounding box grown from
// (f32::MAX, f32::MIN).
SimpleMesh load_stl(const std::string &path);

// match_meshes (src/inputs.rs:95-129): the space-separated file names of one argument,
// dispatched on the lower-cased extension.
std::vector<SimpleMesh> match_meshes(const std::string &files);

// The reference's Context on one GPU.
class Context {
public:
    explicit Context(bool image, int device = 0);
    ~Context();
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;

    size_t width = 0, height = 0;
    bool image;

    // Context::update for image contexts: utransform from the meshes' bounding boxes.
    void update(const std::vector<SimpleMesh> &meshes);
    // Context::clear.
    void clear();
    // draw_mesh(context, mesh, transform, default_shader); the mesh is uploaded on first use.
    void draw_mesh(const SimpleMesh &mesh, const float transform[16]);
    // Context::flush(color, webify): the same bytes, written to `out`.
    void flush(bool color, bool webify, std::FILE *out);
    // The frame (char | r<<8 | g<<16 | b<<24 per cell) and depth buffers.
    void read(std::vector<uint32_t> *cells, std::vector<float> *z);

private:
    sloth_ctx *ctx_ = nullptr;
    std::map<const SimpleMesh *, sloth_mesh *> uploaded_;
    std::vector<char> text_;
    void check(sloth_status st, const char *what);
};

}  // namespace sloth_host
