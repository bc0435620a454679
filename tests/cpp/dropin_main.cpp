// A host program written against the reference's ParticleSystem interface
// (gpu/src/particlesystem.h), built with include/particle_system.hpp and
// libpbd_gb300.so: the reference's constructor, scene builders, runtime
// insertion and update loop, then a check of the result and of the render
// buffer copy.
#include <cmath>
#include <cstdio>

#include "particle_system.hpp"

int main() {
    // the reference app's constants (particleapp.cpp:23-38)
    pbd::ParticleSystem ps(0.25f, make_uint3(64, 64, 64), 20000, make_int3(-50, 0, -50), make_int3(50, 200, 50), 5);
    ps.addFluid(make_int3(-3, 0, -3), make_int3(3, 4, 3), 1.f, 1.f, make_float3(0.f, 0.f, 1.f));
    ps.addRope(make_float3(-6.f, 20.f, 0.f), make_float3(0.45f, -0.12f, 0.05f), 0.4f, 16, 1.f, true);
    ps.addHorizCloth(make_int2(5, -3), make_int2(10, 2), make_float3(0.5f, 7.f, 0.5f), make_float2(0.5f, 0.5f), 1.f,
                     true);
    const unsigned n0 = ps.getNumParticles();
    ps.setParticleToAdd(make_float3(0.f, 12.f, 0.f), make_float3(0.f, -5.f, 0.f), 1.f);
    ps.setFluidToAdd(make_float3(1.f, 9.f, 1.f), make_float3(0.f, 0.f, 1.f), 1.f, 1.f);
    for (int k = 0; k < 30; ++k) ps.update(1.f / 60.f);
    const unsigned n1 = ps.getNumParticles();
    std::vector<float4> p = ps.getPositions();
    int bad = 0;
    for (const float4 &q : p)
        if (!std::isfinite(q.x) || !std::isfinite(q.y) || !std::isfinite(q.z) || q.y < -1e-3f || q.y > 200.f) ++bad;
    // the render buffer a renderer written for the reference reads
    float4 *vbo = nullptr;
    cudaMalloc((void **)&vbo, p.size() * sizeof(float4));
    ps.copyVbo(vbo);
    std::vector<float4> r(p.size());
    cudaMemcpy(r.data(), vbo, r.size() * sizeof(float4), cudaMemcpyDeviceToHost);
    cudaFree(vbo);
    for (size_t k = 0; k < p.size(); ++k)
        if (r[k].x != p[k].x || r[k].y != p[k].y || r[k].z != p[k].z || r[k].w != 1.f) ++bad;
    bool threw = false;
    try {
        ps.makeDistanceConstraint(make_uint2(0, 1000000), 1.f);  // no such particle
    } catch (const pbd::Error &e) {
        threw = e.code == PBD_ERR_INVALID_ARGUMENT;
    }
    std::printf("n0 %u n1 %u bad %d threw %d\n", n0, n1, bad, threw ? 1 : 0);
    return (n1 == n0 + 2 && bad == 0 && threw) ? 0 : 1;
}
