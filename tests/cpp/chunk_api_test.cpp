// Uses the C++ chunk interface the way the reference's World and boids use
// chunk::Chunk (world.rs:113-145, boid.rs:130-207), and dumps what it got for
// tests/test_cpp_host.py to compare with the CPU oracle.
//   chunk_api_test <dump file>
#include <cstdio>
#include <cstring>
#include <vector>

#include "uww_chunk.hpp"

using namespace uww_host;

static void put(FILE* f, const void* p, size_t bytes)
{
    const unsigned long long n = bytes;
    fwrite(&n, sizeof(n), 1, f);
    if (bytes) fwrite(p, 1, bytes, f);
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    try {
        Perlin perlin(0);  // noise::Perlin::new(0), reference constants
        std::vector<Pos> positions;
        for (int x = -2; x <= 2; ++x)
            for (int y = -2; y <= 2; ++y)
                for (int z = -2; z <= 2; ++z) positions.push_back({x, y, z});
        std::vector<Chunk> chunks = build_chunks(perlin, positions);

        // the one-chunk path gives the same chunk as the batch
        int mismatches = 0;
        for (size_t i : {size_t(62), size_t(37), size_t(88)}) {
            Chunk c(positions[i]);
            if (!c.build_partial(perlin)) ++mismatches;
            if (c.not_blank() != chunks[i].not_blank() || c.num_inds() != chunks[i].num_inds()) ++mismatches;
            if (c.inds() != chunks[i].inds()) ++mismatches;
            if (c.verts().size() != chunks[i].verts().size() ||
                (c.verts().size() && std::memcmp(c.verts().data(), chunks[i].verts().data(),
                                                 c.verts().size() * sizeof(uww_vert_color))))
                ++mismatches;
        }
        if (mismatches) {
            std::fprintf(stderr, "plain and batched builds differ (%d)\n", mismatches);
            return 1;
        }
        // an empty list builds nothing
        if (!build_chunks(perlin, {}).empty()) {
            std::fprintf(stderr, "an empty list gave chunks\n");
            return 1;
        }

        FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 3;
        const unsigned long long n = chunks.size();
        fwrite(&n, sizeof(n), 1, f);
        for (const Chunk& c : chunks) {
            const unsigned char nb = c.not_blank();
            fwrite(&nb, 1, 1, f);
            put(f, c.verts().data(), c.verts().size() * sizeof(uww_vert_color));
            put(f, c.inds().data(), c.inds().size() * sizeof(uint32_t));
            std::vector<uint16_t> u16 = c.inds_u16();
            put(f, u16.data(), u16.size() * sizeof(uint16_t));
            // tris_around at three points inside the chunk, WALL_RANGE = 3 (boid.rs:15)
            std::vector<float> tri_data;
            for (const Vec3& lp : {Vec3{0.5f, 0.5f, 0.5f}, Vec3{0.1f, 0.8f, 0.3f}, Vec3{0.95f, 0.05f, 0.6f}}) {
                std::vector<Tri> tris = c.tris_around(lp, 3);
                tri_data.push_back((float)tris.size());
                for (const Tri& t : tris) {
                    for (const Vec3& v : t.verts) tri_data.insert(tri_data.end(), v.begin(), v.end());
                    tri_data.insert(tri_data.end(), t.normal.begin(), t.normal.end());
                }
            }
            put(f, tri_data.data(), tri_data.size() * sizeof(float));
        }
        // perlin_util::iso_at at a few points in chunk units
        std::vector<Vec3> pts = {{0.1f, 0.2f, 0.3f}, {-1.5f, 2.25f, 0.75f}, {1.0f, -1.0f, -1.9f}};
        std::vector<float> iso = iso_at(perlin, pts);
        put(f, pts.data(), pts.size() * sizeof(Vec3));
        put(f, iso.data(), iso.size() * sizeof(float));
        std::fclose(f);
    } catch (const Error& e) {
        std::fprintf(stderr, "uww error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
