// uww_chunk.hpp -- C++ mirror of the reference's Rust chunk-build interface
// over the C ABI of libuww_gb300.so (include/uww.h).
//
// Reference (LelsersLasers/UnderwaterWorld, underwater_world/src/):
//   noise::Perlin::new(seed)                  (state.rs:359)         -> Perlin
//   perlin_util::iso_at                       (perlin_util.rs:24-29) -> iso_at
//   chunk::Chunk::new / build_full / build_partial (chunk.rs:89-103, 266-313)
//   Chunk::not_blank / num_inds / buffer slices    (chunk.rs:344-348)
//   Chunk::tris_around                        (chunk.rs:315-342)     -> Chunk::tris_around
//   util::Tri::new / Tri::intersects          (util.rs:12-58)        -> Tri
//   World's per-frame chunk builds            (world.rs:113-145)     -> build_chunks (one batched launch)
//
// The reference's chunk code returns no errors (blank is None, internal
// failures panic); here a failing library call throws uww_host::Error with
// the library's status.  Everything runs on the GPU through the C ABI; there
// is no CPU fallback.
#pragma once

#include <array>
#include <cstdint>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "uww.h"

namespace uww_host {

constexpr int32_t CHUNK_SIZE = 16;     // chunk.rs:5
constexpr int32_t INTERNAL_SIZE = 12;  // chunk.rs:6

using Pos = std::array<int32_t, 3>;
using Vec3 = std::array<float, 3>;

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what);
    int status;
};

// noise::Perlin plus the world's density parameters, bound to one CUDA
// context of the library.  Defaults: the reference constants (chunk.rs:5-17,
// perlin_util.rs:6-29) with this seed; vertex colours and per-cell cases (the
// latter for tris_around) are produced.
class Perlin {
public:
    explicit Perlin(uint32_t seed);
    explicit Perlin(const uww_params& params);
    ~Perlin();
    Perlin(const Perlin&) = delete;
    Perlin& operator=(const Perlin&) = delete;

    uww_ctx* ctx() const { return ctx_; }
    const uww_params& params() const { return params_; }

private:
    uww_params params_;
    uww_ctx* ctx_ = nullptr;
};

// perlin_util::iso_at(perlin, x, y, z) with (x, y, z) in chunk units
// (world / CHUNK_SIZE, as boid.rs:132-137 calls it).
float iso_at(const Perlin& perlin, float x, float y, float z);
std::vector<float> iso_at(const Perlin& perlin, const std::vector<Vec3>& xyz);

// util::Tri
struct Tri {
    std::array<Vec3, 3> verts;
    Vec3 normal;
    static Tri make(const Vec3& a, const Vec3& b, const Vec3& c);                 // Tri::new
    std::optional<float> intersects(const Vec3& pos, const Vec3& dir, float range) const;
};

class Chunk {
public:
    explicit Chunk(Pos pos, uint32_t cells = INTERNAL_SIZE);  // Chunk::new

    void build_full(const Perlin& perlin);     // one batched launch of one chunk
    bool build_partial(const Perlin& perlin);  // finishes in its first call (the build is one launch)

    bool not_blank() const { return done_ && num_inds() > 0; }
    size_t num_inds() const { return inds_.size(); }
    bool done() const { return done_; }
    Pos pos() const { return pos_; }
    uint32_t cells() const { return cells_; }
    const uww_chunk_record& record() const { return record_; }

    const std::vector<uww_vert_color>& verts() const { return verts_; }  // verts_buffer_slice contents
    const std::vector<uint32_t>& inds() const { return inds_; }
    std::vector<uint16_t> inds_u16() const;                              // inds_buffer_slice as Uint16
    const std::vector<uint8_t>& cases() const { return cases_; }

    // the triangles of the cells within `range` of local_pos_percent
    // (fractions of the chunk along x, y, z)
    std::vector<Tri> tris_around(const Vec3& local_pos_percent, int32_t range) const;

private:
    friend std::vector<Chunk> build_chunks(const Perlin&, const std::vector<Pos>&, uint32_t);
    Pos pos_;
    uint32_t cells_;
    bool done_ = false;
    uww_chunk_record record_{};
    std::vector<uww_vert_color> verts_;
    std::vector<uint32_t> inds_;
    std::vector<uint8_t> cases_;
    std::vector<uint32_t> cell_first_;  // first index of each cell's triangles
};

// Every chunk of the list in one batched build (the reference builds a few
// per frame, world.rs:113-145); chunks come back in the list's order.
std::vector<Chunk> build_chunks(const Perlin& perlin, const std::vector<Pos>& positions,
                                uint32_t cells = INTERNAL_SIZE);

}  // namespace uww_host
