// Drives lc::CudaDeformableBody (include/lc/lc_body.hpp) the way the
// reference's scene code drives Physics::CudaDeformableBody: construct from a
// vertex array, then FixedUpdate() and Update() once per frame.
//
// stdin:  int32 V, int32 T, int32 steps, int32 tune, float[3V] positions,
//         uint32[3T] indices, uint8[V] pinned, lc_cloth_params (raw struct
//         bytes); tune = 1 runs the body's Autotune() (launch shapes only)
//         before the first step
// stdout: float[3V] published positions after the last Update()
#include <cstdint>
#include <cstdio>
#include <vector>

#include "lc/lc_body.hpp"

namespace {
struct Vec3 { float x, y, z; };
// Field layout of Rendering::VertexFormat (position, color, normal, uv).
struct Vertex {
    Vec3 m_position;
    float m_color[4];
    Vec3 m_normal;
    float m_uv[2];
};

template <class T> bool read(T *dst, size_t n) { return std::fread(dst, sizeof(T), n, stdin) == n; }
}  // namespace

int main() {
    int32_t V = 0, T = 0, steps = 0, tune = 0;
    if (!read(&V, 1) || !read(&T, 1) || !read(&steps, 1) || !read(&tune, 1) || V <= 0 || T <= 0) return 2;
    std::vector<float> pos(3 * (size_t)V);
    std::vector<unsigned int> idx(3 * (size_t)T);
    std::vector<uint8_t> pin(V);
    lc_cloth_params params;
    if (!read(pos.data(), pos.size()) || !read(idx.data(), idx.size()) || !read(pin.data(), pin.size()) ||
        !read(&params, 1))
        return 2;
    std::vector<Vertex> verts(V);
    std::vector<bool> fixed(V);
    for (int i = 0; i < V; ++i) {
        verts[i].m_position = Vec3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        fixed[i] = pin[i] != 0;
    }
    try {
        lc::CudaDeformableBody<Vertex> body(&verts, &idx, params, fixed);
        if (tune) body.Autotune(2, 1, false);
        for (int s = 0; s < steps; ++s) {
            body.FixedUpdate();
            body.Update();
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    for (int i = 0; i < V; ++i) std::fwrite(&verts[i].m_position, sizeof(float), 3, stdout);
    return 0;
}
