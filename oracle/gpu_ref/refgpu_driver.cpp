/*
 * refgpu_driver.cpp -- runs the reference's own GPU kernels and thrust
 * functors (gpu/src/cuda/integration_kernel.cuh, solver_kernel.cuh,
 * included from the reference tree in place) on the CPU, in the order of
 * the reference's host wrappers (gpu/src/cuda/integration.cu,
 * solver.cu) and ParticleSystem::update (gpu/src/particlesystem.cpp:
 * 144-246).  Test infrastructure only: built into oracle/_ref/ to pin the
 * oracle restatement against the reference code itself.
 *
 * The wrapper bodies are re-expressed here (they need GL interop, cudaMalloc
 * and texture binding, none of which exist on the host): every kernel runs
 * as one-thread blocks over the index range, textures are pointer wrappers
 * bound to the same arrays the reference binds, thrust runs on the host
 * system, and the six cuRAND uniforms per iteration are an input.
 */
#include "integration_kernel.cuh"
#include "solver_kernel.cuh"

#include <thrust/execution_policy.h>
#include <thrust/for_each.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/reduce.h>
#include <thrust/sort.h>
#include <thrust/transform.h>

#include <cstdint>
#include <cstring>
#include <vector>

dim3 blockIdx, blockDim, threadIdx;
uint sharedHash[2];  // blockDim.x + 1 entries for one-thread blocks

namespace {

template <class K>
void launch(uint n, K &&kernel) {
    blockDim = dim3(1, 1, 1);
    threadIdx = dim3(0, 0, 0);
    for (uint b = 0; b < n; ++b) {
        blockIdx = dim3(b, 0, 0);
        kernel();
    }
}

struct RefSys {
    SimParams sp;
    int3 minB, maxB;
    int iterations;
    uint n = 0;
    std::vector<float4> pos, vel, xstar, sortedPos, posCopy;
    std::vector<float> W, sortedW, ros, lambda;
    std::vector<int> phase, sortedPhase;
    std::vector<uint> hash, index, cellStart, cellEnd, neighbors, numNeighbors;
    // constraints (solver.cu:32-41)
    std::vector<uint> distsI, pointsI, sortedI, occurences;
    std::vector<float> dists, points;
    std::vector<float4> deltas;
    float rands[6] = {0, 0, 0, 0, 0, 0};
};

void bind_params(RefSys *s) { params = s->sp; }

}  // namespace

extern "C" {

RefSys *refgpu_create(float radius, uint gx, uint gy, uint gz, const int *minB, const int *maxB, int iterations) {
    RefSys *s = new RefSys();
    // ParticleSystem::ParticleSystem (particlesystem.cpp:36-69)
    s->sp.gridSize = make_uint3(gx, gy, gz);
    s->sp.numCells = gx * gy * gz;
    s->sp.numBodies = 0;
    s->sp.particleRadius = radius;
    s->sp.worldOrigin = make_float3(0.f, 0.f, 0.f);
    float cellSize = radius * 2.0f;
    s->sp.cellSize = make_float3(cellSize, cellSize, cellSize);
    s->sp.gravity = make_float3(0.0f, -9.8f, 0.0f);
    s->sp.globalDamping = 1.0f;
    s->minB = make_int3(minB[0], minB[1], minB[2]);
    s->maxB = make_int3(maxB[0], maxB[1], maxB[2]);
    s->iterations = iterations;
    s->cellStart.assign(s->sp.numCells, 0xffffffffu);
    s->cellEnd.assign(s->sp.numCells, 0u);
    return s;
}

void refgpu_destroy(RefSys *s) { delete s; }

// addParticleMultiple + appendIntegrationParticle + appendPhaseAndMass +
// appendSolverParticle (particlesystem.cpp:333-348, integration.cu:50-72,
// shared_variables.cu:71-89, solver.cu:64-70).
void refgpu_add_particles(RefSys *s, uint n, const float *pos4, const float *vel4, const float *w,
                          const float *ros, const int *phase) {
    for (uint i = 0; i < n; ++i) {
        s->pos.push_back(make_float4(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]));
        s->vel.push_back(make_float4(vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2], vel4[4 * i + 3]));
        s->W.push_back(w[i]);
        s->ros.push_back(ros[i]);
        s->phase.push_back(phase[i]);
        s->occurences.push_back(0u);
    }
    s->n += n;
    const uint N = s->n;
    s->xstar.resize(N);
    s->sortedPos.resize(N);
    s->sortedW.resize(N);
    s->sortedPhase.resize(N);
    s->hash.resize(N);
    s->index.resize(N);
    s->lambda.resize(N, 0.f);
    s->numNeighbors.resize(N, 0u);
    s->neighbors.resize((size_t)N * MAX_FLUID_NEIGHBORS, 0u);
}

// updateOccurences (solver.cu:72-106).
static void update_occurences(RefSys *s, const uint *index, uint num) {
    std::vector<uint> idx(index, index + num), keys(num), ones(num, 1u);
    thrust::sort(thrust::host, idx.begin(), idx.end());
    auto e = thrust::reduce_by_key(thrust::host, idx.begin(), idx.end(), ones.begin(), keys.begin(), ones.begin());
    uint *occ = s->occurences.data();
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(keys.begin(), ones.begin())),
                     thrust::make_zip_iterator(thrust::make_tuple(e.first, e.second)), occurence_functor(occ));
}

// addPointConstraint (solver.cu:108-123).
void refgpu_add_points(RefSys *s, uint num, const uint *index, const float *pts) {
    s->pointsI.insert(s->pointsI.end(), index, index + num);
    s->points.insert(s->points.end(), pts, pts + 3 * num);
    update_occurences(s, index, num);
}

// addDistanceConstraint (solver.cu:125-156).
void refgpu_add_distances(RefSys *s, uint num, const uint *index, const float *dist) {
    s->dists.insert(s->dists.end(), dist, dist + num);
    s->distsI.insert(s->distsI.end(), index, index + 2 * num);
    s->sortedI.resize(s->distsI.size());
    s->deltas.resize(2 * s->dists.size());
    update_occurences(s, index, 2 * num);
}

void refgpu_set_rands(RefSys *s, const float *r) { std::memcpy(s->rands, r, sizeof s->rands); }

// integrateSystem (integration.cu:122-135).
void refgpu_integrate(RefSys *s, float dt) {
    bind_params(s);
    s->xstar = s->pos;  // copyToXstar
    float4 *p = s->pos.data(), *v = s->vel.data();
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(p, v)),
                     thrust::make_zip_iterator(thrust::make_tuple(p + s->n, v + s->n)), integrate_functor(dt));
}

// calcHash + sortParticles + reorderDataAndFindCellStart
// (integration.cu:161-275).
void refgpu_grid(RefSys *s) {
    bind_params(s);
    const uint n = s->n;
    uint *h = s->hash.data(), *ix = s->index.data();
    float4 *pos = s->pos.data();
    launch(n, [&] { calcHashD(h, ix, pos, n); });
    thrust::sort_by_key(thrust::host, h, h + n, ix);
    std::fill(s->cellStart.begin(), s->cellStart.end(), 0xffffffffu);
    s->posCopy = s->pos;  // the reference copies pos before binding it
    oldPosTex.ptr = s->posCopy.data();
    invMassTex.ptr = s->W.data();
    oldPhaseTex.ptr = s->phase.data();
    uint *cs = s->cellStart.data(), *ce = s->cellEnd.data();
    float4 *sp = s->sortedPos.data();
    float *sw = s->sortedW.data();
    int *sph = s->sortedPhase.data();
    float *W = s->W.data();
    int *ph = s->phase.data();
    launch(n, [&] { reorderDataAndFindCellStartD(cs, ce, sp, sw, sph, h, ix, pos, W, ph, n); });
}

static void bind_sorted(RefSys *s) {
    oldPosTex.ptr = s->sortedPos.data();
    invMassTex.ptr = s->sortedW.data();
    oldPhaseTex.ptr = s->sortedPhase.data();
    cellStartTex.ptr = s->cellStart.data();
    cellEndTex.ptr = s->cellEnd.data();
}

// collide (integration.cu:338-386).
void refgpu_collide(RefSys *s) {
    bind_params(s);
    bind_sorted(s);
    const uint n = s->n;
    float4 *p = s->pos.data(), *xs = s->xstar.data(), *sp = s->sortedPos.data();
    float *sw = s->sortedW.data();
    int *sph = s->sortedPhase.data();
    uint *ix = s->index.data(), *cs = s->cellStart.data(), *ce = s->cellEnd.data();
    uint *nb = s->neighbors.data(), *nn = s->numNeighbors.data();
    launch(n, [&] { collideD(p, xs, sp, sw, sph, ix, cs, ce, n, nb, nn); });
}

// solveFluids (integration.cu:453-508).
void refgpu_solve_fluids(RefSys *s) {
    bind_params(s);
    bind_sorted(s);
    const uint n = s->n;
    float *lam = s->lambda.data(), *ros = s->ros.data();
    uint *ix = s->index.data(), *cs = s->cellStart.data(), *ce = s->cellEnd.data();
    uint *nb = s->neighbors.data(), *nn = s->numNeighbors.data();
    float4 *p = s->pos.data();
    launch(n, [&] { findLambdasD(lam, ix, cs, ce, n, nb, nn, ros); });
    launch(n, [&] { solveFluidsD(lam, ix, p, n, nb, nn, ros); });
}

// collideWorld (integration.cu:319-336), uniforms given.
void refgpu_collide_world(RefSys *s) {
    bind_params(s);
    float4 *p = s->pos.data(), *xs = s->xstar.data();
    int *ph = s->phase.data();
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(p, xs, ph)),
                     thrust::make_zip_iterator(thrust::make_tuple(p + s->n, xs + s->n, ph + s->n)),
                     collide_world_functor(s->rands, s->minB, s->maxB));
}

// solveDistanceConstraints (solver.cu:196-231), including its
// segment-to-particle indexing (solver.cu:227-230).
void refgpu_solve_distances(RefSys *s) {
    const uint m = (uint)s->dists.size();
    if (!m) return;
    float4 *p = s->pos.data();
    uint2 *idx = (uint2 *)s->distsI.data();
    float *d = s->dists.data();
    uint *s1 = s->sortedI.data(), *s2 = s1 + m;
    float4 *d1 = s->deltas.data(), *d2 = d1 + m;
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(idx, d, s1, s2, d1, d2)),
                     thrust::make_zip_iterator(thrust::make_tuple(idx + m, d + m, s1 + m, s2 + m, d1 + m, d2 + m)),
                     delta_computing_functor(p));
    thrust::sort_by_key(thrust::host, s1, s1 + 2 * m, d1);
    auto e = thrust::reduce_by_key(thrust::host, s1, s1 + 2 * m, d1, s1, d1);
    uint size = (uint)(e.first - s1);
    uint *occ = s->occurences.data();
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(p, d1, occ)),
                     thrust::make_zip_iterator(thrust::make_tuple(p + size, d1 + size, occ + size)),
                     distance_constraint_functor());
}

// solvePointConstraints (solver.cu:180-194).
void refgpu_solve_points(RefSys *s) {
    const uint np = (uint)s->pointsI.size();
    if (!np) return;
    uint *ix = s->pointsI.data();
    float3 *pts = (float3 *)s->points.data();
    thrust::for_each(thrust::host, thrust::make_zip_iterator(thrust::make_tuple(ix, pts)),
                     thrust::make_zip_iterator(thrust::make_tuple(ix + np, pts + np)),
                     point_constraint_functor(s->pos.data()));
}

// calcVelocity (integration.cu:416-426).
void refgpu_calc_velocity(RefSys *s, float dt) {
    thrust::transform(thrust::host, s->pos.begin(), s->pos.begin() + s->n, s->xstar.begin(), s->vel.begin(),
                      subtract_functor(dt));
}

// ParticleSystem::update (particlesystem.cpp:144-246) without the GL map
// and the queued-particle insertion.
void refgpu_update(RefSys *s, float dt) {
    dt = std::min(dt, .05f);
    if (s->n == 0) return;
    refgpu_integrate(s, dt);
    for (int i = 0; i < s->iterations; ++i) {
        refgpu_grid(s);
        refgpu_collide(s);
        refgpu_solve_fluids(s);
        refgpu_collide_world(s);
        refgpu_solve_distances(s);
        refgpu_solve_points(s);
    }
    refgpu_calc_velocity(s, dt);
}

uint refgpu_num_particles(RefSys *s) { return s->n; }
void refgpu_get_positions(RefSys *s, float *out) { std::memcpy(out, s->pos.data(), s->n * sizeof(float4)); }
void refgpu_get_velocities(RefSys *s, float *out) { std::memcpy(out, s->vel.data(), s->n * sizeof(float4)); }
void refgpu_set_positions(RefSys *s, const float *in) { std::memcpy(s->pos.data(), in, s->n * sizeof(float4)); }
void refgpu_get_grid(RefSys *s, uint *sorted_hash, uint *sorted_index, uint *cell_start, uint *cell_end) {
    std::memcpy(sorted_hash, s->hash.data(), s->n * 4);
    std::memcpy(sorted_index, s->index.data(), s->n * 4);
    std::memcpy(cell_start, s->cellStart.data(), s->cellStart.size() * 4);
    std::memcpy(cell_end, s->cellEnd.data(), s->cellEnd.size() * 4);
}
// lambda is indexed by sorted slot in the reference
void refgpu_get_lambdas_sorted(RefSys *s, float *out) { std::memcpy(out, s->lambda.data(), s->n * 4); }
void refgpu_get_num_neighbors_sorted(RefSys *s, uint *out) { std::memcpy(out, s->numNeighbors.data(), s->n * 4); }

}  // extern "C"
