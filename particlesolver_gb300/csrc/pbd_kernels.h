// Host-side launchers of the PBD kernels (implemented in pbd_kernels.cu).
// All launchers are asynchronous on the given stream and return the launch
// error (cudaSuccess when the launch was accepted).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbd_device.cuh"

namespace pbd {

// Device arrays of one system's particle state and neighbour grid.
struct GridBuffers {
    uint32_t *hash;        // [cap] cell hash of each particle (original order)
    uint32_t *slot;        // [cap] arrival slot inside its cell
    uint32_t *cell_first;  // [num_cells + 1] counts, then dense offsets
    uint32_t *scan_part;   // [scan partial sums]
    uint32_t *tmp;         // [cap] unstable cell-bucketed indices
    uint32_t *sorted_idx;  // [cap] original index of each sorted slot
    float4 *sorted_x;      // [cap] positions (xyz, w) in sorted order
    SortedAttr *sorted_attr;  // [cap] phase and rest density, sorted
};

// Per-iteration fluid neighbour lists: sorted indices in the reference's
// visiting order, four per uint4, slot-major.  The lambda pass's walk first
// records them as row chunks: chunk (b, m) stands for the sorted slots
// b .. b + 31 of one stencil row, bit k of m set when slot b + k is a
// neighbour; the chunks a particle's walk does not keep in shared memory
// go to `chunk`.
struct NbList {
    uint4 *slot;        // [capacity / 4][stride]
    uint32_t *count;    // [stride] neighbours (low 16 bits), chunks (high 16 bits); 0xffff0000: no list
    uint32_t capacity;  // neighbours per particle, a multiple of 4
    uint32_t stride;    // particles per slot row
    uint2 *chunk;       // [chunks][stride]
    uint32_t chunks;    // chunks per particle
    // Skin lists (reused by later iterations; all null / 0 when off): the
    // list radius is (1 + skin) h; sref holds the sorted positions it was
    // built from; *reuse (set on the device each iteration) selects
    // filtering the old list over a new walk; *ovf records a list that
    // could not be kept (over capacity or the neighbour cap).
    float skin;
    float4 *sref;
    const uint32_t *reuse;
    uint32_t *ovf;
    // Where the lambda pass keeps a list's first chunks while it walks:
    // 0 = shared memory, 1 = none (every chunk stored straight to the
    // global list).
    uint32_t assemble;
};

// Per-particle arrays of the gas phase (all null in a system without gas
// particles).
struct GasBuffers {
    const int *phase;      // [cap] original order
    float4 *force;         // [cap] original order: force the next prediction applies
    const uint8_t *open;   // [cap] original order: 1 = open gas
    float *lam;            // [cap] sorted order: gas lambda
    float4 *v;             // [cap] original order: the step's velocity v' (set by the prediction)
    const uint32_t *sidx;  // [cap] sorted slot -> original index
};

// Signed-distance data of rigid-body particles (all null without any).
struct RigidSdf {
    const float4 *sdf;   // [cap] original order: rest-frame unit normal xyz, depth (< 0: none)
    const int *body;     // [cap] original order: body of the particle, -1 for none
    const float4 *quat;  // [bodies] current rotation of each body (xyzw)
};

// Device words of the skin-list schedule: [0] reuse, [1] overflow, [2 + k]
// largest displacement / h since the list build, seen in iteration k (k <
// kSkinWords - 3), [kSkinWords - 1] iterations of the step that reused.
constexpr uint32_t kSkinWords = 64;

struct ConstraintBuffers {
    uint32_t count;        // constrained particles
    uint32_t *particle;    // [count] particle index
    uint32_t *row;         // [count + 1] CSR rows into the incidence list
    uint32_t *other;       // [incidences] other endpoint
    float *rest;           // [incidences] rest length
    float *stiff;          // [incidences] stiffness
    float *occ;            // [count] constraints touching the particle
    float4 *pin;           // [count] pin point, w = 1 when pinned
    float4 *tmp;           // [count] new positions
    bool any_distance, any_pin;
    // per distance constraint, in add order (stiffness updates, adjoint)
    uint32_t m;            // constraints
    uint32_t *con_a, *con_b;  // [m] endpoints
    float *con_rest, *con_stiff;  // [m]
    uint32_t *inc_con;     // [incidences] constraint of each incidence
    float *occ_of;         // [particles] constraint count of each particle (0: none)
};

struct BodyBuffers {
    uint32_t count;        // bodies
    uint4 *range;          // [count] first particle, particle count, rest offset
    float *stiff;          // [count]
    float4 *rest;          // [rigid particles] rest offset xyz, mass
    float4 *quat;          // [count] rotation of the last solve (x, y, z, w)
};

size_t scan_partial_count(uint32_t elements);

cudaError_t launch_predict(const DevParams &P, uint32_t n, float dt, float4 *x, float4 *v,
                           float4 *x_old, uint32_t *hash, uint32_t *slot, uint32_t *counts,
                           cudaStream_t s, const GasBuffers &gas = GasBuffers{});
cudaError_t launch_hash_count(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash,
                              uint32_t *slot, uint32_t *counts, cudaStream_t s);
// counts[0..cells] -> exclusive offsets; counts[cells] must be zero on entry.
cudaError_t launch_exclusive_scan(uint32_t *data, uint32_t elements, uint32_t *partials,
                                  cudaStream_t s, const uint32_t *skip = nullptr);
// skip: device word; when nonzero the kernels return at once (a reused
// skin list keeps the previous grid).  nullptr = always run.
cudaError_t launch_grid_finish(const DevParams &P, uint32_t n, const GridBuffers &g,
                               const float4 *x, const int *phase, const float *rho0,
                               cudaStream_t s, const uint32_t *skip = nullptr);
// The grid build of a later iteration under the skin-list schedule: clear
// the counts, hash and count -- each skipped when *skip is set.
cudaError_t launch_grid_begin(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash, uint32_t *slot,
                              uint32_t *counts, const uint32_t *skip, cudaStream_t s);
// Skin-list check of iteration `iter`: refreshes the sorted positions from
// x and records the largest displacement / h since the list build in
// words[2 + iter]; then decides words[0] (reuse) from it and words[1].
cudaError_t launch_skin_check(const DevParams &P, uint32_t n, uint32_t iter, float skin, const GridBuffers &g,
                              const float4 *x, const float4 *sref, uint32_t *words, cudaStream_t s);
// The whole grid build into caller buffers: cell hashes, counting sort in
// (hash, index) order, and the reference's cellStart / cellEnd layout.
// hash, slot, tmp: [n]; cell_first: [cells + 1]; partials:
// [scan_partial_count(cells + 1)]; sorted_idx: [n]; cell_start/end: [cells].
cudaError_t launch_sort_into_cells(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash, uint32_t *slot,
                                   uint32_t *cell_first, uint32_t *partials, uint32_t *tmp, uint32_t *sorted_idx,
                                   uint32_t *cell_start, uint32_t *cell_end, cudaStream_t s);
cudaError_t launch_refresh_sorted(uint32_t n, const GridBuffers &g, const float4 *x,
                                  cudaStream_t s);
// The whole grid build of a small single-scene system in one block of 1024
// threads (cell counts, scan, bucket, stable rank and reorder in shared
// memory; the same result as the multi-kernel build): n <= kSmallGridN and
// small_grid_smem(num_cells, n) <= kSmallGridSmem.  One launch instead of
// six and a memset per build.
constexpr uint32_t kSmallGridN = 8192;
constexpr size_t kSmallGridSmem = 200u * 1024u;
size_t small_grid_smem(uint32_t num_cells, uint32_t n);
cudaError_t launch_grid_small(const DevParams &P, uint32_t n, const GridBuffers &g, const float4 *x,
                              const int *phase, const float *rho0, cudaStream_t s);
// tpp: lanes sharing one particle's neighbour walk (1, 2, 4, 8, 16, 32).
// sxl: per sorted slot (position xyz, lambda) -- written by the lambda pass,
// read by the solve pass.
// With tpp == 1 and a list allocated, the lambda pass also records the
// neighbour list that the solve and XSPH passes then use (use_list).
//
// P.table set: a batched launch over every scene of a system, each slot
// taking its scene's parameters.  iter_left: solver iterations still to come
// in the step after this one (a scene with K iterations is active while
// iter_left < K); the single-stage entry points pass 0.
cudaError_t launch_lambda(const DevParams &P, uint32_t n, uint32_t iter_left, const GridBuffers &g, float4 *sxl,
                          const NbList &L, uint32_t tpp, cudaStream_t s, const GasBuffers &gas = GasBuffers{});
cudaError_t launch_solve(const DevParams &P, uint32_t n, uint32_t mask, uint32_t iter_left, const GridBuffers &g,
                         const float4 *sxl, const float4 *x_old, float4 *x, const NbList &L, bool use_list,
                         uint32_t tpp, cudaStream_t s, const GasBuffers &gas = GasBuffers{},
                         const RigidSdf &sdf = RigidSdf{});
cudaError_t launch_distance(const DevParams &P, uint32_t iter_left, const ConstraintBuffers &c, float4 *x,
                            bool apply_distance, bool apply_pins, cudaStream_t s);
cudaError_t launch_shapes(const DevParams &P, uint32_t iter_left, const BodyBuffers &b, float4 *x, cudaStream_t s);
// dt is clamped to each scene's max_dt on the device (predict and velocity).
cudaError_t launch_velocity(const DevParams &P, uint32_t n, float dt, const float4 *x, const float4 *x_old,
                            float4 *v, cudaStream_t s);
// vs: scratch for the velocities in sorted order.  With x (and x_old, dt)
// the velocity update is fused in: the gather computes each particle's
// velocity as launch_velocity does and writes it to v as well, so that
// launch_velocity is not needed first.
cudaError_t launch_xsph(const DevParams &P, uint32_t n, const GridBuffers &g, float4 *v, float4 *vs,
                        const NbList &L, bool use_list, uint32_t tpp, cudaStream_t s, float dt = 0.f,
                        const float4 *x = nullptr, const float4 *x_old = nullptr);
// Solidification of the fluid emitter over the sorted slots of the last grid.
cudaError_t launch_solidify(uint32_t n, float dt, float speed, float height, const uint32_t *sidx, const float4 *sxl,
                            const uint8_t *tag, float *timer, float4 *x, float4 *x_old, float4 *v, int *phase,
                            float4 *force, uint32_t *converted, uint32_t *list, cudaStream_t s);
cudaError_t launch_finite_check(uint32_t n, const float4 *x, const float4 *v, uint32_t *flag,
                                cudaStream_t s);
// dst[k] = (x[k].xyz, 1): the reference's render buffer layout.
cudaError_t launch_vbo(uint32_t n, const float4 *x, float4 *dst, cudaStream_t s);

}  // namespace pbd
