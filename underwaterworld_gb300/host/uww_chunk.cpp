// uww_chunk.cpp -- implementation of the C++ chunk interface (uww_chunk.hpp).
// Built with -ffp-contract=off: Tri::make and Tri::intersects follow
// util.rs:12-58 in f32 with every operation separately rounded, as Rust
// (cgmath) computes them.
#include "uww_chunk.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "mc_tables.h"

namespace uww_host {

namespace {

void check(int status, const char* what)
{
    if (status != UWW_OK) {
        std::string msg = std::string(what) + ": " + uww_status_string(status);
        const char* last = uww_last_error();
        if (last && *last) msg += std::string(" [") + last + "]";
        throw Error(status, msg);
    }
}

Vec3 sub(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
float dot(const Vec3& a, const Vec3& b)
{
    float r = a[0] * b[0];
    r = r + a[1] * b[1];
    return r + a[2] * b[2];
}
Vec3 cross(const Vec3& a, const Vec3& b)
{
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
// util::safe_normalize (util.rs:61-64)
Vec3 safe_normalize(const Vec3& v)
{
    const float mag = std::sqrt(dot(v, v));
    if (mag == 0.f) return v;
    return {v[0] / mag, v[1] / mag, v[2] / mag};
}

// per-cell first index of its triangles: stream order, 3 * ntri(case) each
std::vector<uint32_t> cell_first(const std::vector<uint8_t>& cases)
{
    std::vector<uint32_t> f(cases.size());
    uint32_t run = 0;
    for (size_t i = 0; i < cases.size(); ++i) {
        f[i] = run;
        run += 3u * UWW_CASE_NTRI[cases[i]];
    }
    return f;
}

}  // namespace

Error::Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}

Perlin::Perlin(uint32_t seed)
{
    uww_params_reference(&params_);
    params_.seed = seed;
    params_.outputs = UWW_OUT_COLOR | UWW_OUT_CASES;
    check(uww_ctx_create(&params_, nullptr, &ctx_), "uww_ctx_create");
}

Perlin::Perlin(const uww_params& params) : params_(params)
{
    params_.outputs |= UWW_OUT_CASES;
    check(uww_ctx_create(&params_, nullptr, &ctx_), "uww_ctx_create");
}

Perlin::~Perlin()
{
    if (ctx_) uww_ctx_destroy(ctx_);
}

std::vector<float> iso_at(const Perlin& perlin, const std::vector<Vec3>& xyz)
{
    std::vector<float> out(xyz.size());
    if (xyz.empty()) return out;
    // world coordinates, device buffers
    std::vector<float> w(3 * xyz.size());
    for (size_t i = 0; i < xyz.size(); ++i)
        for (int j = 0; j < 3; ++j) w[3 * i + j] = xyz[i][j] * (float)CHUNK_SIZE;
    void* d_in = nullptr;
    void* d_out = nullptr;
    check(uww_device_alloc(w.size() * sizeof(float), &d_in), "uww_device_alloc");
    int st = uww_device_alloc(out.size() * sizeof(float), &d_out);
    if (st == UWW_OK) st = uww_memcpy(perlin.ctx(), d_in, w.data(), w.size() * sizeof(float), 0);
    if (st == UWW_OK) st = uww_density_at(perlin.ctx(), (const float*)d_in, (uint32_t)xyz.size(), (float*)d_out);
    if (st == UWW_OK) st = uww_memcpy(perlin.ctx(), out.data(), d_out, out.size() * sizeof(float), 1);
    if (st == UWW_OK) st = uww_ctx_sync(perlin.ctx());
    uww_device_free(d_in);
    if (d_out) uww_device_free(d_out);
    check(st, "iso_at");
    return out;
}

float iso_at(const Perlin& perlin, float x, float y, float z) { return iso_at(perlin, std::vector<Vec3>{{x, y, z}})[0]; }

Tri Tri::make(const Vec3& a, const Vec3& b, const Vec3& c)
{
    Tri t;
    t.verts = {a, b, c};
    t.normal = safe_normalize(cross(sub(b, a), sub(c, a)));
    return t;
}

std::optional<float> Tri::intersects(const Vec3& pos, const Vec3& dir, float range) const
{
    const float dn = dot(normal, dir);
    if (std::fabs(dn) < 1e-5f) return std::nullopt;
    const float t = dot(normal, sub(verts[0], pos)) / dn;
    if (t < 0.f || t > range) return std::nullopt;
    const Vec3 p = {pos[0] + dir[0] * t, pos[1] + dir[1] * t, pos[2] + dir[2] * t};
    const float d0 = dot(cross(sub(verts[1], verts[0]), sub(p, verts[0])), normal);
    const float d1 = dot(cross(sub(verts[2], verts[1]), sub(p, verts[1])), normal);
    const float d2 = dot(cross(sub(verts[0], verts[2]), sub(p, verts[2])), normal);
    if (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f) return t;
    return std::nullopt;
}

Chunk::Chunk(Pos pos, uint32_t cells) : pos_(pos), cells_(cells) {}

void Chunk::build_full(const Perlin& perlin)
{
    std::vector<Chunk> one = build_chunks(perlin, {pos_}, cells_);
    *this = std::move(one[0]);
}

bool Chunk::build_partial(const Perlin& perlin)
{
    if (!done_) build_full(perlin);
    return true;
}

std::vector<uint16_t> Chunk::inds_u16() const
{
    std::vector<uint16_t> r(inds_.size());
    for (size_t i = 0; i < inds_.size(); ++i) {
        if (inds_[i] > 0xFFFFu) throw Error(UWW_ERR_INVALID_ARG, "chunk has more than 65536 vertices");
        r[i] = (uint16_t)inds_[i];
    }
    return r;
}

std::vector<Tri> Chunk::tris_around(const Vec3& p, int32_t range) const
{
    std::vector<Tri> tris;
    if (!not_blank()) return tris;
    const int N = (int)cells_;
    const int mx = (int)std::floor(p[0] * (float)N), my = (int)std::floor(p[1] * (float)N),
              mz = (int)std::floor(p[2] * (float)N);
    const int x0 = std::max(mx - range, 0), y0 = std::max(my - range, 0), z0 = std::max(mz - range, 0);
    const int x1 = std::min(mx + range, N - 1), y1 = std::min(my + range, N - 1), z1 = std::min(mz + range, N - 1);
    for (int x = x0; x <= x1; ++x)
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) {
                const size_t c = (size_t)((x * N + y) * N + z);
                const int nt = UWW_CASE_NTRI[cases_[c]];
                for (int j = 0; j < nt; ++j) {
                    Vec3 v[3];
                    for (int m = 0; m < 3; ++m) {
                        const uww_vert_color& vc = verts_[inds_[cell_first_[c] + 3 * j + m]];
                        v[m] = {vc.pos[0], vc.pos[1], vc.pos[2]};
                    }
                    tris.push_back(Tri::make(v[0], v[1], v[2]));
                }
            }
    return tris;
}

std::vector<Chunk> build_chunks(const Perlin& perlin, const std::vector<Pos>& positions, uint32_t cells)
{
    const uint32_t n = (uint32_t)positions.size();
    if (n == 0) return {};
    std::vector<uww_chunk_desc> desc(n);
    for (uint32_t i = 0; i < n; ++i) {
        std::memset(&desc[i], 0, sizeof(desc[i]));
        for (int j = 0; j < 3; ++j) desc[i].pos[j] = positions[i][j];
        desc[i].cells = cells;
    }
    uint64_t total_cells = 0;
    check(uww_layout_cells(desc.data(), n, &total_cells, nullptr), "uww_layout_cells");
    std::vector<uww_chunk_record> rec(n);
    std::vector<uint8_t> cases(total_cells);
    uint64_t totals[4] = {0, 0, 0, 0};
    // a first guess at the capacities; on UWW_ERR_CAPACITY the totals hold the
    // sizes needed, and the batch is rebuilt once with them
    uint64_t vcap = std::max<uint64_t>(1024, (uint64_t)n * 512), icap = 3 * vcap;
    std::vector<uww_vert_color> verts;
    std::vector<uint32_t> inds;
    for (int attempt = 0;; ++attempt) {
        verts.resize(vcap);
        inds.resize(icap);
        uww_mesh_out out;
        std::memset(&out, 0, sizeof(out));
        out.verts = verts.data();
        out.inds = inds.data();
        out.cases = cases.data();
        out.case_capacity = total_cells;
        out.records = rec.data();
        out.totals = totals;
        out.vert_capacity = (uint32_t)vcap;
        out.ind_capacity = (uint32_t)icap;
        const int st = uww_build_chunks_host(perlin.ctx(), desc.data(), n, &out);
        if (st == UWW_ERR_CAPACITY && attempt == 0) {
            vcap = totals[0] + 1;
            icap = totals[1] + 1;
            continue;
        }
        check(st, "uww_build_chunks_host");
        break;
    }
    std::vector<Chunk> chunks;
    chunks.reserve(n);
    const size_t nc = (size_t)cells * cells * cells;
    for (uint32_t i = 0; i < n; ++i) {
        Chunk c(positions[i], cells);
        c.record_ = rec[i];
        c.verts_.assign(verts.begin() + rec[i].vert_offset, verts.begin() + rec[i].vert_offset + rec[i].num_verts);
        c.inds_.assign(inds.begin() + rec[i].ind_offset, inds.begin() + rec[i].ind_offset + rec[i].num_inds);
        c.cases_.assign(cases.begin() + desc[i].cell_offset, cases.begin() + desc[i].cell_offset + nc);
        c.cell_first_ = cell_first(c.cases_);
        c.done_ = true;
        chunks.push_back(std::move(c));
    }
    return chunks;
}

}  // namespace uww_host
