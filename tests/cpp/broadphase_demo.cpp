// Drives lc::CollisionMethod (include/lc/lc_body.hpp) as scene code drives
// Collision::ICollisionMethod: reads int32 method, n, frames, then n boxes
// (6 floats each), from stdin; adds the objects (ids 100 + i), then for each
// frame moves every third object by +0.01 on x and removes the object with
// the highest id, runs Update() and TestCollision(), and writes the frame's
// pair count and pairs (int32 ids, lower first) to stdout.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "lc/lc_body.hpp"

int main() {
    int32_t head[3];
    if (std::fread(head, sizeof(head), 1, stdin) != 1) return 2;
    const int method = head[0], n = head[1], frames = head[2];
    std::vector<float> box(6 * (size_t)n);
    if (n && std::fread(box.data(), sizeof(float), box.size(), stdin) != box.size()) return 2;
    lc_broadphase_desc d{};
    d.method = method;
    d.max_objects = n;
    for (int k = 0; k < 3; ++k) { d.world_min[k] = 0.f; d.world_max[k] = 1.f; }
    d.cells_per_axis = 16;
    d.cell_size = 0.05f;
    d.table_size = 4096;
    try {
        lc::CollisionMethod<int> m(d);
        for (int i = 0; i < n; ++i) m.ObjectAdded(100 + i, &box[6 * (size_t)i], &box[6 * (size_t)i + 3]);
        int top = 100 + n - 1;
        for (int f = 0; f < frames; ++f) {
            for (int i = 0; i < n; i += 3) {
                if (100 + i > top) break;
                box[6 * (size_t)i] += 0.01f;
                box[6 * (size_t)i + 3] += 0.01f;
                m.ObjectMoved(100 + i, &box[6 * (size_t)i], &box[6 * (size_t)i + 3]);
            }
            m.ObjectRemoved(top--);
            m.Update();
            const auto pairs = m.TestCollision();
            const int32_t cnt = (int32_t)pairs.size();
            std::fwrite(&cnt, sizeof(cnt), 1, stdout);
            for (const auto &p : pairs) {
                const int32_t ab[2] = {p.first < p.second ? p.first : p.second, p.first < p.second ? p.second : p.first};
                std::fwrite(ab, sizeof(ab), 1, stdout);
            }
            if (m.GetLastFrameCriteria().count("Intersection Tests") != 1) return 3;
        }
    } catch (const lc::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
