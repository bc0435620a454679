// Scene builders of the reference ParticleSystem class
// (gpu/src/particlesystem.cpp:357-687), producing the same lattices,
// constraints and phases on the host and appending them through the C ABI.
// Jitter comes from a seeded splitmix64 stream instead of rand().
#include <cmath>
#include <cstdint>
#include <vector>

#include "pbd_system.h"

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    // uniform in [-1, 1)
    float sym() { return (float)((double)(next() >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0); }
};

// (int)ceil(ur - ll) / spacing, truncated, as the reference computes its
// lattice counts (particlesystem.cpp:363,416,465,621).
int lattice_count(int lo, int hi, float spacing) {
    return (int)((float)(int)std::ceil((float)(hi - lo)) / spacing);
}

bool is_twod(const pbd_system *s) { return (s->cur_params().flags & PBD_FLAG_TWOD) != 0u; }

int add_block(pbd_system *s, const int32_t ll[3], const int32_t ur[3], float distance, float jitter,
              float w, float ro, int phase, uint64_t seed) {
    if (!ll || !ur) return PBD_ERR_INVALID_ARGUMENT;
    const int cx = lattice_count(ll[0], ur[0], distance), cy = lattice_count(ll[1], ur[1], distance);
    const int cz = is_twod(s) ? 1 : lattice_count(ll[2], ur[2], distance);
    if (cx <= 0 || cy <= 0 || cz <= 0) return PBD_OK;
    SplitMix64 rng{seed};
    const size_t count = (size_t)cx * cy * cz;
    std::vector<float> pos(4 * count);
    std::vector<int32_t> ph(count, phase);
    std::vector<float> rho(count, ro);
    size_t k = 0;
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x, ++k) {
                pos[4 * k + 0] = ll[0] + x * distance + rng.sym() * jitter;
                pos[4 * k + 1] = ll[1] + y * distance + rng.sym() * jitter;
                pos[4 * k + 2] = is_twod(s) ? s->cur_params().twod_z : ll[2] + z * distance + rng.sym() * jitter;
                pos[4 * k + 3] = w;
            }
    uint32_t first;
    return pbd_add_particles(s, (uint32_t)count, pos.data(), nullptr, ph.data(), rho.data(), &first);
}

}  // namespace

extern "C" {

int pbd_add_fluid(pbd_system *s, const int32_t ll[3], const int32_t ur[3], float mass, float density,
                  uint64_t seed) {
    if (!s) return PBD_ERR_INVALID_ARGUMENT;
    if (!(mass > 0.f) || !(density > 0.f)) return PBD_ERR_INVALID_ARGUMENT;
    const float r = s->cur_params().particle_radius;
    return add_block(s, ll, ur, r * 2.5f, r * 0.01f, 1.f / mass, density, PBD_PHASE_FLUID, seed);
}

int pbd_add_particle_grid(pbd_system *s, const int32_t ll[3], const int32_t ur[3], float mass, int jitter,
                          uint64_t seed) {
    if (!s) return PBD_ERR_INVALID_ARGUMENT;
    if (!(mass > 0.f)) return PBD_ERR_INVALID_ARGUMENT;
    const float r = s->cur_params().particle_radius;
    return add_block(s, ll, ur, r * 2.002f, jitter ? r * 0.01f : 0.f, 1.f / mass, 1.f, PBD_PHASE_SOLID, seed);
}

int pbd_add_horiz_cloth(pbd_system *s, const int32_t ll[2], const int32_t ur[2], const float spacing[3],
                        const float dist[2], float mass, int hold_edges) {
    if (!s || !ll || !ur || !spacing || !dist || !(mass > 0.f)) return PBD_ERR_INVALID_ARGUMENT;
    const int cx = lattice_count(ll[0], ur[0], spacing[0]);
    const int cy = lattice_count(ll[1], ur[1], spacing[2]);
    if (cx <= 0 || cy <= 0) return PBD_OK;
    const uint32_t start = s->n;
    const size_t count = (size_t)cx * cy;
    std::vector<float> pos(4 * count), pts;
    std::vector<uint32_t> pairs, pin;
    std::vector<float> rest;
    std::vector<int32_t> ph(count, PBD_PHASE_RIGID + s->rigid_index);
    size_t k = 0;
    for (int z = 0; z < cy; ++z)
        for (int x = 0; x < cx; ++x, ++k) {
            pos[4 * k + 0] = ll[0] + x * spacing[0];
            pos[4 * k + 1] = spacing[1];
            pos[4 * k + 2] = is_twod(s) ? s->cur_params().twod_z : ll[1] + z * spacing[2];
            pos[4 * k + 3] = 1.f / mass;
            const uint32_t pidx = start + (uint32_t)(z * cx + x);
            auto add_pin = [&]() {
                pin.push_back(pidx);
                pts.insert(pts.end(), {pos[4 * k + 0], pos[4 * k + 1], pos[4 * k + 2]});
            };
            if (x > 0) {
                pairs.insert(pairs.end(), {pidx - 1u, pidx});
                rest.push_back(dist[0]);
            } else {
                add_pin();
            }
            if (z > 0) {
                pairs.insert(pairs.end(), {pidx - (uint32_t)cx, pidx});
                rest.push_back(dist[1]);
            } else if (hold_edges) {
                add_pin();
            }
            if (x == cx - 1 && hold_edges) add_pin();
            if (z == cy - 1 && hold_edges) add_pin();
        }
    uint32_t first;
    int rc = pbd_add_particles(s, (uint32_t)count, pos.data(), nullptr, ph.data(), nullptr, &first);
    if (rc) return rc;
    rc = pbd_add_point_constraints(s, (uint32_t)pin.size(), pin.data(), pts.data());
    if (rc) return rc;
    rc = pbd_add_distance_constraints(s, (uint32_t)rest.size(), pairs.data(), rest.data(), nullptr);
    if (rc) return rc;
    ++s->rigid_index;
    return PBD_OK;
}

int pbd_add_rope(pbd_system *s, const float start[3], const float spacing[3], float dist, int32_t links,
                 float mass, int pin_start) {
    if (!s || !start || !spacing || links < 1 || !(mass > 0.f)) return PBD_ERR_INVALID_ARGUMENT;
    const uint32_t first_idx = s->n;
    const size_t count = (size_t)links + 1;
    std::vector<float> pos(4 * count);
    std::vector<uint32_t> pairs;
    std::vector<float> rest;
    std::vector<int32_t> ph(count, PBD_PHASE_RIGID + s->rigid_index);
    for (size_t i = 0; i < count; ++i) {
        pos[4 * i + 0] = start[0] + (float)i * spacing[0];
        pos[4 * i + 1] = start[1] + (float)i * spacing[1];
        pos[4 * i + 2] = start[2] + (float)i * spacing[2];
        pos[4 * i + 3] = 1.f / mass;
        if (i > 0) {
            pairs.insert(pairs.end(), {first_idx + (uint32_t)i - 1u, first_idx + (uint32_t)i});
            rest.push_back(dist);
        }
    }
    uint32_t first;
    int rc = pbd_add_particles(s, (uint32_t)count, pos.data(), nullptr, ph.data(), nullptr, &first);
    if (rc) return rc;
    rc = pbd_add_distance_constraints(s, (uint32_t)rest.size(), pairs.data(), rest.data(), nullptr);
    if (rc) return rc;
    if (pin_start) {
        rc = pbd_add_point_constraints(s, 1, &first_idx, start);
        if (rc) return rc;
    }
    ++s->rigid_index;
    return PBD_OK;
}

int pbd_add_static_sphere(pbd_system *s, const int32_t ll[3], const int32_t ur[3], float spacing) {
    if (!s || !ll || !ur || !(spacing > 0.f)) return PBD_ERR_INVALID_ARGUMENT;
    const int cx = lattice_count(ll[0], ur[0], spacing), cy = lattice_count(ll[1], ur[1], spacing);
    const int cz = is_twod(s) ? 1 : lattice_count(ll[2], ur[2], spacing);
    const float radius = (float)(ur[0] - ll[0]) * .5f;
    const float c[3] = {(float)ll[0] + radius, (float)ll[1] + radius, (float)ll[2] + radius};
    std::vector<float> pos, pts;
    std::vector<uint32_t> idx;
    const uint32_t start = s->n;
    for (int z = 0; z < cz; ++z)
        for (int y = 0; y < cy; ++y)
            for (int x = 0; x < cx; ++x) {
                const float p[3] = {ll[0] + x * spacing, ll[1] + y * spacing,
                                    is_twod(s) ? s->cur_params().twod_z : ll[2] + z * spacing};
                const float dx = p[0] - c[0], dy = p[1] - c[1], dz = p[2] - c[2];
                if (std::sqrt(dx * dx + dy * dy + dz * dz) < radius) {
                    pos.insert(pos.end(), {p[0], p[1], p[2], .01f});  // W = .01 (particlesystem.cpp:675)
                    idx.push_back(start + (uint32_t)idx.size());
                    pts.insert(pts.end(), {p[0], p[1], p[2]});
                }
            }
    if (idx.empty()) return PBD_OK;
    std::vector<int32_t> ph(idx.size(), PBD_PHASE_RIGID + s->rigid_index);
    uint32_t first;
    int rc = pbd_add_particles(s, (uint32_t)idx.size(), pos.data(), nullptr, ph.data(), nullptr, &first);
    if (rc) return rc;
    rc = pbd_add_point_constraints(s, (uint32_t)idx.size(), idx.data(), pts.data());
    if (rc) return rc;
    ++s->rigid_index;
    return PBD_OK;
}

}  // extern "C"
