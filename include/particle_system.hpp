// particle_system.hpp -- drop-in C++ ParticleSystem over the pbd.h C ABI.
//
// Same public methods, argument meanings and call order as the reference
// class (gpu/src/particlesystem.h:22-53); differences:
//   * no OpenGL: positions live in a device buffer (devicePositions()) or
//     are copied out with getPositions(); getCurrentReadBuffer() is gone;
//   * errors throw pbd::Error instead of exiting or being ignored;
//   * update() takes an optional cudaStream_t.
// Header-only; link with libpbd_gb300.so.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pbd.h"

namespace pbd {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &what) : std::runtime_error(what), code(c) {}
};

class ParticleSystem {
  public:
    // ParticleSystem(particleRadius, gridSize, maxParticles, minBounds,
    // maxBounds, iterations) (particlesystem.cpp:36-69): cell size 2 r,
    // world origin 0, gravity (0, -9.8, 0), reference PBF constants.
    ParticleSystem(float particleRadius, uint3 gridSize, unsigned maxParticles, int3 minBounds,
                   int3 maxBounds, int iterations) {
        pbd_params p;
        pbd_default_params(&p);
        p.particle_radius = particleRadius;
        p.cell_size = particleRadius * 2.f;
        p.grid_size[0] = gridSize.x;
        p.grid_size[1] = gridSize.y;
        p.grid_size[2] = gridSize.z;
        p.box_min[0] = (float)minBounds.x; p.box_min[1] = (float)minBounds.y; p.box_min[2] = (float)minBounds.z;
        p.box_max[0] = (float)maxBounds.x; p.box_max[1] = (float)maxBounds.y; p.box_max[2] = (float)maxBounds.z;
        p.iterations = (uint32_t)iterations;
        check(pbd_create(&p, maxParticles, &sys_), nullptr);
        minB_ = minBounds;
        maxB_ = maxBounds;
        radius_ = particleRadius;
    }
    explicit ParticleSystem(const pbd_params &p, unsigned maxParticles) {
        check(pbd_create(&p, maxParticles, &sys_), nullptr);
        radius_ = p.particle_radius;
        minB_ = make_int3((int)p.box_min[0], (int)p.box_min[1], (int)p.box_min[2]);
        maxB_ = make_int3((int)p.box_max[0], (int)p.box_max[1], (int)p.box_max[2]);
    }
    ~ParticleSystem() {
        if (sys_) pbd_destroy(sys_);
    }
    ParticleSystem(const ParticleSystem &) = delete;
    ParticleSystem &operator=(const ParticleSystem &) = delete;

    // ParticleSystem::update (particlesystem.cpp:144-246): queued particles
    // join first (addNewStuff), then one step.
    void update(float deltaTime, cudaStream_t stream = nullptr) {
        addNewStuff();
        check(pbd_update(sys_, deltaTime, stream));
    }

    // Runtime insertion (particlesystem.cpp:249-350): queued here, added at
    // the start of the next update().  A "shot" particle is solid (phase
    // PBD_PHASE_SOLID, rest density 1.5) with jitter U(-0.01 r, 0.01 r) on
    // x and y (seeded here; the reference used rand()); a fluid particle
    // starts with velocity (0, -1, 0).  The reference silently dropped
    // particles past capacity; here update() throws pbd::Error.
    void setParticleToAdd(float3 pos, float3 vel, float mass) {
        const float j = radius_ * 0.01f;
        pos.x += (uniform() * 2.f - 1.f) * j;
        pos.y += (uniform() * 2.f - 1.f) * j;
        queue(pos, vel, mass, 1.5f, PBD_PHASE_SOLID);
    }
    void setFluidToAdd(float3 pos, float3 /*color*/, float mass, float density) {
        queue(pos, make_float3(0.f, -1.f, 0.f), mass, density, PBD_PHASE_FLUID);
    }
    void addNewStuff() {
        if (add_phase_.empty()) return;
        const uint32_t n = (uint32_t)add_phase_.size();
        const int rc = pbd_add_particles(sys_, n, add_pos_.data(), add_vel_.data(), add_phase_.data(),
                                         add_rho_.data(), nullptr);
        add_pos_.clear();
        add_vel_.clear();
        add_phase_.clear();
        add_rho_.clear();
        check(rc);
    }

    void addFluid(int3 ll, int3 ur, float mass, float density, float3 /*color*/) {
        const int32_t a[3] = {ll.x, ll.y, ll.z}, b[3] = {ur.x, ur.y, ur.z};
        check(pbd_add_fluid(sys_, a, b, mass, density, seed_++));
    }
    void addParticleGrid(int3 ll, int3 ur, float mass, bool addJitter) {
        const int32_t a[3] = {ll.x, ll.y, ll.z}, b[3] = {ur.x, ur.y, ur.z};
        check(pbd_add_particle_grid(sys_, a, b, mass, addJitter ? 1 : 0, seed_++));
    }
    void addHorizCloth(int2 ll, int2 ur, float3 spacing, float2 dist, float mass, bool holdEdges) {
        const int32_t a[2] = {ll.x, ll.y}, b[2] = {ur.x, ur.y};
        const float sp[3] = {spacing.x, spacing.y, spacing.z}, d[2] = {dist.x, dist.y};
        check(pbd_add_horiz_cloth(sys_, a, b, sp, d, mass, holdEdges ? 1 : 0));
    }
    void addRope(float3 start, float3 spacing, float dist, int numLinks, float mass, bool constrainStart) {
        const float s[3] = {start.x, start.y, start.z}, sp[3] = {spacing.x, spacing.y, spacing.z};
        check(pbd_add_rope(sys_, s, sp, dist, numLinks, mass, constrainStart ? 1 : 0));
    }
    void addStaticSphere(int3 ll, int3 ur, float spacing) {
        const int32_t a[3] = {ll.x, ll.y, ll.z}, b[3] = {ur.x, ur.y, ur.z};
        check(pbd_add_static_sphere(sys_, a, b, spacing));
    }
    void makePointConstraint(unsigned index, float3 point) {
        const float p[3] = {point.x, point.y, point.z};
        check(pbd_add_point_constraints(sys_, 1, &index, p));
    }
    void makeDistanceConstraint(uint2 index, float distance) {
        const uint32_t pr[2] = {index.x, index.y};
        check(pbd_add_distance_constraints(sys_, 1, pr, &distance, nullptr));
    }

    unsigned getNumParticles() const { return pbd_num_particles(sys_); }
    float getParticleRadius() const { return radius_; }
    int3 getMinBounds() const { return minB_; }
    int3 getMaxBounds() const { return maxB_; }
    // Device float4 positions (the reference's VBO contents).
    // The reference's render buffer content (xyz, w = 1) into dst, float4
    // per particle, device memory, on the stream.
    void copyVbo(float4 *dst, cudaStream_t stream = nullptr) {
        check(pbd_get_vbo(sys_, 0, pbd_num_particles(sys_), (float *)dst, 1, stream));
    }
    float4 *devicePositions() {
        pbd_device_buffers b;
        check(pbd_get_device_buffers(sys_, &b));
        return (float4 *)b.positions;
    }
    std::vector<float4> getPositions() {
        std::vector<float4> out(getNumParticles());
        if (!out.empty()) check(pbd_get_positions(sys_, 0, (uint32_t)out.size(), (float *)out.data(), 0, nullptr));
        return out;
    }
    pbd_system *handle() { return sys_; }

  private:
    void queue(float3 pos, float3 vel, float mass, float rho0, int32_t phase) {
        const float w = 1.f / mass;
        add_pos_.insert(add_pos_.end(), {pos.x, pos.y, pos.z, w});
        add_vel_.insert(add_vel_.end(), {vel.x, vel.y, vel.z, 0.f});
        add_phase_.push_back(phase);
        add_rho_.push_back(rho0);
    }
    // splitmix64 in [0, 1)
    float uniform() {
        uint64_t z = (jitter_ += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (float)((z >> 40) * (1.0 / 16777216.0));
    }
    void check(int rc, const pbd_system *s) const {
        if (rc) throw Error(rc, pbd_last_error(s));
    }
    void check(int rc) const { check(rc, sys_); }

    pbd_system *sys_ = nullptr;
    float radius_ = 0.f;
    int3 minB_{}, maxB_{};
    uint64_t seed_ = 1;
    uint64_t jitter_ = 0x5eedull;
    std::vector<float> add_pos_, add_vel_, add_rho_;
    std::vector<int32_t> add_phase_;
};

}  // namespace pbd
