// Device-side parameter block and shared inline math of the PBD step.
//
// The reference kept SimParams in __constant__ memory, refreshed with
// cudaMemcpyToSymbol every step (integration_kernel.cuh:55,
// integration.cu:96-100), which ties the whole program to one system.  Here
// the block travels by value as a kernel argument: several systems can run
// side by side and a captured CUDA graph carries its own copy.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pbd {

enum : int { kFluid = 0, kGas = 1, kCloth = 2, kSolid = 3, kRigid = 4 };

enum : uint32_t {
    kFlagTwoD = 1u << 0,
    kFlagDensityNeighborMass = 1u << 1,
    kFlagDeltaOverRho0 = 1u << 2,
    kFlagDistanceMassWeighted = 1u << 3,
    kFlagKernelUnits = 1u << 4,
    kFlagSkipFixedNeighbors = 1u << 5,
    kFlagDeltaOverCount = 1u << 6,
    kFlagCpuContacts = 1u << 7,
    // Set by the host, never by the caller: the system holds gas particles,
    // so the prediction applies the per-particle force and the gas gravity
    // and keeps the step's velocity v' for the gas terms.
    kFlagHasGas = 1u << 16,
    // Set by the host: some rigid body carries signed-distance data, so the
    // contact pass looks it up for solid pairs.
    kFlagHasSdf = 1u << 17,
};

// Stage mask of the fused per-particle solve kernel.
enum : uint32_t { kDoContact = 1u, kDoFluid = 2u, kDoWorld = 4u };

// Numeric constants the reference hard-codes (integration_kernel.cuh:20,
// 319, 580, 626; solver_kernel.cuh:57).
constexpr float kEps = 0.001f;           // EPS
constexpr float kCollideScale = 2.001f;  // collideDist = r * 2.001
constexpr float kMinSpiky2 = 1e-8f;      // spiky gradient cut-off |r|^2 < (1e-4)^2
constexpr float kMinDistLen = 0.0001f;   // distance constraint cut-off

struct DevParams {
    float3 gravity;
    float r;             // particle radius
    float h, h2;         // PBF kernel radius and its square
    float cell;          // grid cell edge
    float3 origin;       // grid origin
    uint32_t gx, gy, gz; // cells per axis (powers of two)
    uint32_t num_cells;
    float3 bmin, bmax;   // world box
    float poly6;         // 315 / (64 pi h^9)
    float spiky;         // 45 / (pi h^6)
    float poly6_self;    // poly6 * h^6
    float scorr_k, scorr_n;
    float scorr_inv_ref; // 1 / (poly6 * (h^2 - (dq h)^2)^3)
    int scorr_n_int;     // n when integral (repeated product), else 0
    float relax;
    float xsph_c;
    float cs, ck;        // contact static / kinetic friction
    float ws, wk;        // sqrt of wall static / kinetic friction
    float collide_dist, collide2;
    int fluid_rad;       // ceil(h / cell)
    // Stencil trimming is exact only when no two cells of a stencil alias
    // to one grid cell: 2 rad + 1 <= every grid dimension.
    bool trim_fluid, trim_contact;
    uint32_t max_nb;
    float twod_z;
    int twod_cz;         // z cell of twod_z: in 2-D mode every particle's
                         // grid z (the particles sit in one layer)
    uint32_t flags;
    float solid_w;       // density weight of neighbours of phase >= CLOTH
    float rands[6];      // wall jitter uniforms
    // gas phase (gasconstraint.cpp / .h, simulation.h:21)
    float3 gas_gravity;     // gravity times gas_gravity_scale
    float gas_scorr_k;      // K_P (times h^2 in kernel units)
    float gas_scorr_inv_ref;// 1 / (poly6 * (h^2 - (DQ_P h)^2)^3)
    float gas_solid_w;      // S_SOLID: density weight of phases >= CLOTH
    float gas_drag;         // open gas: force += v (1 - rho / rho0) (-gas_drag)
    uint32_t iterations; // solver iterations per step
    float max_dt;        // step length clamp
    // First cell of this scene in the cell space shared by every scene of a
    // system (0 for a system with one scene): each scene hashes into its own
    // block of cells, so one counting sort keeps scenes apart and contiguous.
    uint32_t cell_base;
    // Batched launches only (nullptr otherwise): the parameter block of every
    // scene and the scene of every particle slot.  A scene's particles
    // occupy the same slot range in original and in sorted order.
    const DevParams *table;
    const uint16_t *scene_of;
};

#if defined(__CUDACC__)
__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ void operator+=(float3 &a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__device__ __forceinline__ void operator-=(float3 &a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }

// Squared distance with a fixed rounding sequence (no contraction choice left
// to the compiler), so that the oracle can reproduce every neighbour test
// bit for bit: d2 = fma(dz, dz, fma(dy, dy, dx * dx)).
__device__ __forceinline__ float dist2_exact(float3 a, float3 b) {
    float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// calcGridPos (integration_kernel.cuh:187-194) with IEEE division and
// floor; the float-to-int conversion saturates (NaN -> 0).
__device__ __forceinline__ int3 grid_pos(const DevParams &P, float3 p) {
    int3 g;
    g.x = __float2int_rd(__fdiv_rn(__fsub_rn(p.x, P.origin.x), P.cell));
    g.y = __float2int_rd(__fdiv_rn(__fsub_rn(p.y, P.origin.y), P.cell));
    g.z = (P.flags & kFlagTwoD) ? P.twod_cz : __float2int_rd(__fdiv_rn(__fsub_rn(p.z, P.origin.z), P.cell));
    return g;
}

// The z offsets a stencil covers: in 2-D mode only the particles' own layer.
__device__ __forceinline__ int stencil_zrad(const DevParams &P, int rad) {
    return (P.flags & kFlagTwoD) ? 0 : rad;
}

// calcGridHash (integration_kernel.cuh:197-203): wrap each coordinate into
// the power-of-two grid, then linearise x fastest.
__device__ __forceinline__ uint32_t grid_hash(const DevParams &P, int3 g) {
    uint32_t x = (uint32_t)g.x & (P.gx - 1u);
    uint32_t y = (uint32_t)g.y & (P.gy - 1u);
    uint32_t z = (uint32_t)g.z & (P.gz - 1u);
    return P.cell_base + (z * P.gy + y) * P.gx + x;
}

// Visits the candidate particles of the (2 rad + 1)^3 cell stencil around
// cell g, in the reference's order (z outer, y, x inner, then ascending
// sorted index; integration_kernel.cuh:388-398, 549-559).  cell_first holds
// num_cells + 1 dense offsets into the sorted arrays, so a stencil row whose
// cells do not wrap is one contiguous index range; a wrapping row falls back
// to per-cell ranges, which also reproduces the double visit of aliased
// cells when the stencil is wider than the grid.  f(j) returns false to
// stop the walk.
template <class F>
__device__ __forceinline__ void for_each_candidate(const DevParams &P, int3 g, int rad,
                                                   const uint32_t *__restrict__ cell_first, F &&f) {
    const int zr = stencil_zrad(P, rad);
    for (int dz = -zr; dz <= zr; ++dz) {
        const uint32_t z = (uint32_t)(g.z + dz) & (P.gz - 1u);
        for (int dy = -rad; dy <= rad; ++dy) {
            const uint32_t y = (uint32_t)(g.y + dy) & (P.gy - 1u);
            const uint32_t row = P.cell_base + (z * P.gy + y) * P.gx;
            const int x0 = g.x - rad, x1 = g.x + rad;
            if (x0 >= 0 && x1 < (int)P.gx) {
                const uint32_t b = __ldg(cell_first + row + (uint32_t)x0);
                const uint32_t e = __ldg(cell_first + row + (uint32_t)x1 + 1u);
                for (uint32_t j = b; j < e; ++j)
                    if (!f(j)) return;
            } else {
                for (int dx = -rad; dx <= rad; ++dx) {
                    const uint32_t c = row + ((uint32_t)(g.x + dx) & (P.gx - 1u));
                    const uint32_t b = __ldg(cell_first + c), e = __ldg(cell_first + c + 1u);
                    for (uint32_t j = b; j < e; ++j)
                        if (!f(j)) return;
                }
            }
        }
    }
}

// Parameters of the scene that slot i belongs to: the launch's own block
// for a single scene, the scene table's entry in a batched launch.
template <bool B>
__device__ __forceinline__ DevParams scene_params(const DevParams &P0, uint32_t i) {
    if constexpr (B) return P0.table[P0.scene_of[i]];
    else return P0;
}

// Iterations run right-aligned in a batch: a scene with K iterations is
// active in the last K of the batch's, so its last iteration (whose grid
// and neighbour lists XSPH reuses) is everyone's last.  iter_left counts
// the batch iterations still to come after the current one.
template <bool B>
__device__ __forceinline__ bool scene_active(const DevParams &P, uint32_t iter_left) {
    return !B || iter_left < P.iterations;
}

#endif  // __CUDACC__

#if defined(__CUDACC__)
// Weight of neighbour j in a fluid particle's density sum and own gradient
// (pbd_params.solid_density_weight for phases >= CLOTH, else 1); the phase
// is only read when the weight is not 1.
template <class AttrPtr>
__device__ __forceinline__ float density_weight(const DevParams &P, AttrPtr sattr, uint32_t j) {
    float w = 1.f;
    if (P.solid_w != 1.f && sattr[j].phase >= kCloth) w = P.solid_w;
    return w;
}
#endif

#if defined(__CUDACC__)
// Whether particle j (sorted position and inverse mass q_j) can be a fluid
// particle's neighbour: always, unless PBD_FLAG_SKIP_FIXED_NEIGHBORS leaves
// fixed particles (w = 0) out (cpu totalfluidconstraint.cpp:59).
__device__ __forceinline__ bool fluid_nb_ok(const DevParams &P, float wj) {
    return !(P.flags & kFlagSkipFixedNeighbors) || wj != 0.f;
}
// The same for a neighbour known by its sorted slot (the inverse mass is
// loaded only when the flag is set).
__device__ __forceinline__ bool fluid_nb_ok_at(const DevParams &P, const float4 *__restrict__ sx, uint32_t j) {
    return !(P.flags & kFlagSkipFixedNeighbors) || __ldg(&sx[j].w) != 0.f;
}
// Divisor of a fluid particle's PBF correction: rho0 + n (the GPU
// reference, integration_kernel.cuh:640), rho0 (PBD_FLAG_DELTA_OVER_RHO0)
// or rho0 (n + 1), the CPU reference's (neighbours + self) rest densities
// (PBD_FLAG_DELTA_OVER_COUNT, totalfluidconstraint.cpp:108,114; its other
// constraints' counts are zero here: fluid takes no part in contacts).
__device__ __forceinline__ float fluid_delta_div(const DevParams &P, float rho0, uint32_t nb) {
    if (P.flags & kFlagDeltaOverCount) return rho0 * (float)(nb + 1u);
    return (P.flags & kFlagDeltaOverRho0) ? rho0 : rho0 + (float)nb;
}
#endif

// Per-particle attributes gathered into sorted order with the positions.
struct __align__(8) SortedAttr {
    int phase;
    float rho0;
};

}  // namespace pbd
