// context.cpp -- the reference's Context and draw_mesh over the C ABI.
#include <cstring>
#include <string>

#include "sloth_host.hpp"

namespace sloth_host {

Context::Context(bool image_mode, int device) : image(image_mode)
{
    check(sloth_ctx_create(&ctx_, device, nullptr), "sloth_ctx_create");
}

Context::~Context()
{
    for (auto &kv : uploaded_) sloth_mesh_destroy(kv.second);
    sloth_ctx_destroy(ctx_);
}

void Context::check(sloth_status st, const char *what)
{
    if (st != SLOTH_OK)
        throw std::runtime_error(std::string(what) + ": " + (ctx_ ? sloth_ctx_last_error(ctx_) : "no context"));
}

// Context::update (src/context.rs:93-141) for image contexts: the viewport is the
// context's own width and height, the scale comes from the meshes' bounding boxes.
void Context::update(const std::vector<SimpleMesh> &meshes)
{
    if (width == 0 && height == 0) return;   // terminal_size == old_size: nothing changes
    std::vector<float> bb;
    for (const SimpleMesh &m : meshes) bb.insert(bb.end(), m.bbox_max, m.bbox_max + 3);
    float u[16];
    sloth_viewport_transform((uint16_t)width, (uint16_t)height, sloth_scene_extent(bb.data(), (uint32_t)meshes.size()),
                             u);
    check(sloth_ctx_set_utransform(ctx_, u), "sloth_ctx_set_utransform");
}

void Context::clear()
{
    if (width == 0 || height == 0) return;   // empty buffers: nothing on the device
    check(sloth_ctx_set_viewport(ctx_, (uint32_t)width, (uint32_t)height, image ? 1 : 0), "sloth_ctx_set_viewport");
    check(sloth_ctx_clear(ctx_), "sloth_ctx_clear");
}

void Context::draw_mesh(const SimpleMesh &mesh, const float transform[16])
{
    if (width == 0 || height == 0 || mesh.triangles() == 0) return;
    auto it = uploaded_.find(&mesh);
    if (it == uploaded_.end()) {
        sloth_mesh *m = nullptr;
        check(sloth_mesh_create(ctx_, mesh.x.data(), mesh.y.data(), mesh.z.data(), (uint32_t)mesh.x.size(), nullptr,
                                (uint32_t)mesh.triangles(), mesh.rgb.data(), mesh.bbox_max, &m),
              "sloth_mesh_create");
        it = uploaded_.emplace(&mesh, m).first;
    }
    check(sloth_draw_mesh(ctx_, it->second, transform), "sloth_draw_mesh");
}

// Context::flush (src/context.rs:50-92): the bytes are formatted on the GPU.
void Context::flush(bool color, bool webify, std::FILE *out)
{
    const int format = !color ? SLOTH_FLUSH_PLAIN : (webify ? SLOTH_FLUSH_HTML : SLOTH_FLUSH_ANSI);
    if (width == 0 || height == 0) {
        // an empty frame: only the cursor move of a terminal context and println's newline
        if (!image) std::fputs("\x1b[1;1H", out);
        if (format == SLOTH_FLUSH_PLAIN) std::fputc('\n', out);
        return;
    }
    uint64_t n = 0;
    check(sloth_ctx_flush(ctx_, format, nullptr, 0, &n), "sloth_ctx_flush");
    text_.resize(n ? n : 1);
    check(sloth_ctx_flush(ctx_, format, text_.data(), n, &n), "sloth_ctx_flush");
    std::fwrite(text_.data(), 1, n, out);
}

void Context::read(std::vector<uint32_t> *cells, std::vector<float> *z)
{
    const size_t nz = width * height, nc = image ? nz + height : nz;
    if (cells) cells->assign(nc, (uint32_t)' ');
    if (z) z->assign(nz, 3.40282347e38f);
    if (nz == 0) return;
    check(sloth_ctx_read(ctx_, cells ? cells->data() : nullptr, z ? z->data() : nullptr, nullptr), "sloth_ctx_read");
}

}  // namespace sloth_host
