// sm_103a kernels of the unified PBD step: prediction, the neighbour grid
// (cell hash, stable counting sort into cells, reorder into sorted SoA,
// dense cell offsets), the PBF density/lambda solve, contacts with friction,
// world walls, distance constraints and pins as a per-particle gather,
// shape matching with a 3x3 rotation extraction, the velocity update and
// XSPH.  Reference kernels are cited beside each replacement.
#include "pbd_kernels.h"

#include <cfloat>
#include <cmath>
#include <utility>

namespace pbd {

namespace {

constexpr int kBlock = 256;

// Compile-time shapes of the neighbour passes (measured on the 1M dam
// break; a build may override them): candidates per unrolled step of the
// list build's walk, list quads whose gathers are in flight together in
// the delta pass, and the minimum resident blocks of the fused solve
// kernel with one lane per particle: its full form (PBF delta, contacts,
// walls) and its contact-and-wall form for batches without fluid
// (0 = no register cap).
#ifndef PBD_WALK_UNROLL
#define PBD_WALK_UNROLL 4
#endif
#ifndef PBD_DELTA_QUADS
#define PBD_DELTA_QUADS 1
#endif
#ifndef PBD_SOLVE_MIN_BLOCKS
#define PBD_SOLVE_MIN_BLOCKS 5
#endif
#ifndef PBD_CONTACT_MIN_BLOCKS
#define PBD_CONTACT_MIN_BLOCKS 8
#endif
#ifndef PBD_LAMBDA_MIN_BLOCKS
#define PBD_LAMBDA_MIN_BLOCKS 6
#endif
// The batched list build reads each slot's parameter block (76 registers
// uncapped): capped at 64 for 8 blocks per SM (512-scene batch: 49,060 ->
// 50,017 scenes*steps/s).
#ifndef PBD_BATCH_LAMBDA_MIN_BLOCKS
#define PBD_BATCH_LAMBDA_MIN_BLOCKS 8
#endif
#ifndef PBD_BATCH_SOLVE_MIN_BLOCKS
#define PBD_BATCH_SOLVE_MIN_BLOCKS 4
#endif
constexpr int kWalkUnroll = PBD_WALK_UNROLL;
// Block of the shared-memory list build, and the row chunks per particle
// it keeps in shared memory (further chunks go straight to the global
// list): columns x kListBlock uint2.  A particle at rest density with cells
// of h has about nine rows with neighbours, one chunk each; skin lists,
// whose rows are longer, get more.  Fewer columns leave more of the SM's
// combined L1/shared storage to cache the candidates the walk loads.
#ifndef PBD_SLIST_COLS
#define PBD_SLIST_COLS 12
#endif
constexpr int kListBlock = 128;
constexpr uint32_t kSharedListCols = PBD_SLIST_COLS;
constexpr uint32_t kSharedListColsSkin = 20;
static_assert(kSharedListCols <= kSharedListColsSkin && kSharedListColsSkin * kListBlock * 8 <= 48 * 1024,
              "shared-memory list build exceeds the default dynamic shared memory");
// NbList::assemble: kListShared selects the shared-memory build (any other
// value: chunks stored straight to the global list).
constexpr uint32_t kListShared = 0u;

inline unsigned blocks_for(uint32_t n, int per_block = kBlock) {
    return (unsigned)((n + (uint32_t)per_block - 1u) / (uint32_t)per_block);
}

// Programmatic dependent launch.  The step's kernels are launched with
// pdl_launch; pdl_launch<true> (the grid build's short kernels) lets a
// kernel be scheduled while its predecessor in the stream is still
// running.  Each of these kernels starts with pdl_entry(): it waits there
// until the predecessor has completed and its writes are visible, and then
// allows its own successor to be scheduled (once every one of its blocks
// has got that far), so launch latencies and prologues overlap the
// predecessors' last waves.  A kernel launched the usual way
// (pdl_launch<false>) passes pdl_entry() at once.  Measured on the 1M dam
// break: eager grid builds 0.249 -> 0.200 ms per step; in graph replay the
// grid kernels gain nothing measurable, and early launch of the long
// per-particle passes cost 1.5 %, so those are launched the usual way.
#ifndef PBD_PDL
#define PBD_PDL 1
#endif
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <bool PDL = true, typename... KArgs, typename... Args>
inline void pdl_launch(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                       Args &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = PDL && PBD_PDL;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---------------------------------------------------------------- predict

// integrate_functor + copyToXstar (integration_kernel.cuh:159-184,
// shared_variables.cu:91-96): x_old = x; v' = v + g dt; x += v' dt.  The
// reference does not store v'; neither do we (the velocity is recomputed
// from positions at the end of the step).  When counts is given, the cell
// hash of the predicted position is computed and counted here too, which is
// the first grid build's calcHashD (integration_kernel.cuh:206-225).  The
// step is min(dt, max_dt) of the particle's scene.  In a system with gas
// (kFlagHasGas) the step's velocity is the CPU reference's (simulation.cpp:
// 142-153): v' = v + dt g' + dt f, with g' = gravity * gas_gravity_scale for
// gas particles and f the force the gas terms accumulated in the last step,
// which is cleared; v' is stored for the gas terms of this step (the final
// velocity update overwrites it).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_predict(DevParams P0, uint32_t n, float dt_in,
                                                    float4 *__restrict__ x,
                                                    float4 *__restrict__ v,
                                                    float4 *__restrict__ x_old,
                                                    uint32_t *__restrict__ hash,
                                                    uint32_t *__restrict__ slot,
                                                    uint32_t *__restrict__ counts,
                                                    GasBuffers gas) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    const float dt = fminf(dt_in, P.max_dt);
    float4 p = x[i];
    const float4 vel = v[i];
    x_old[i] = p;
    float3 vv;
    if (P.flags & kFlagHasGas) {
        const float3 g = gas.phase[i] == kGas ? P.gas_gravity : P.gravity;
        const float3 f = f3(gas.force[i]);
        gas.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        // v + dt g' + dt f with the rounding fixed (the same in every
        // instantiation of this kernel)
        vv = make_float3(__fmaf_rn(f.x, dt, __fmaf_rn(g.x, dt, vel.x)), __fmaf_rn(f.y, dt, __fmaf_rn(g.y, dt, vel.y)),
                         __fmaf_rn(f.z, dt, __fmaf_rn(g.z, dt, vel.z)));
        v[i] = make_float4(vv.x, vv.y, vv.z, vel.w);
    } else {
        vv = make_float3(vel.x, vel.y, vel.z) + P.gravity * dt;
    }
    p.x += vv.x * dt;
    p.y += vv.y * dt;
    p.z += vv.z * dt;
    x[i] = p;
    if (counts) {
        const uint32_t h = grid_hash(P, grid_pos(P, f3(p)));
        hash[i] = h;
        slot[i] = atomicAdd(counts + h, 1u);
    }
}

// calcHashD (integration_kernel.cuh:206-225) plus the per-cell count of the
// counting sort.  The arrival slot is only used to bucket indices; the final
// order inside a cell is fixed by original index in k_rank_reorder.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_hash_count(DevParams P0, uint32_t n,
                                                       const float4 *__restrict__ x,
                                                       uint32_t *__restrict__ hash,
                                                       uint32_t *__restrict__ slot,
                                                       uint32_t *__restrict__ counts,
                                                       const uint32_t *__restrict__ skip) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (skip && *skip)) return;
    const DevParams P = scene_params<B>(P0, i);
    const uint32_t h = grid_hash(P, grid_pos(P, f3(x[i])));
    hash[i] = h;
    slot[i] = atomicAdd(counts + h, 1u);
}

// ------------------------------------------------------------------- scan

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Exclusive scan of one value per thread over a 1024-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *smem,
                                                         uint32_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive_scan(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t s = warp_inclusive_scan(smem[lane]);
        smem[lane] = s;
    }
    __syncthreads();
    const uint32_t prefix = warp ? smem[warp - 1] : 0u;
    total = smem[31];
    __syncthreads();
    return prefix + inc - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t *__restrict__ data,
                                                              uint32_t elements,
                                                              uint32_t *__restrict__ partials,
                                                              const uint32_t *__restrict__ skip) {
    pdl_entry();
    if (skip && *skip) return;
    __shared__ uint32_t smem[32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < elements) s += data[base + k];
    uint32_t total;
    block_exclusive_scan(s, smem, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partials(uint32_t *__restrict__ partials,
                                                                uint32_t count,
                                                                const uint32_t *__restrict__ skip) {
    pdl_entry();
    if (skip && *skip) return;
    __shared__ uint32_t smem[32];
    uint32_t carry = 0;
    for (uint32_t chunk = 0; chunk < count; chunk += kScanTile) {
        const uint32_t base = chunk + threadIdx.x * kScanItems;
        uint32_t v[kScanItems], s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = (base + k < count) ? partials[base + k] : 0u;
            s += v[k];
        }
        uint32_t total;
        uint32_t run = carry + block_exclusive_scan(s, smem, total);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (base + k < count) partials[base + k] = run;
            run += v[k];
        }
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(uint32_t *__restrict__ data,
                                                             uint32_t elements,
                                                             const uint32_t *__restrict__ partials,
                                                             const uint32_t *__restrict__ skip) {
    pdl_entry();
    if (skip && *skip) return;
    __shared__ uint32_t smem[32];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < elements) ? data[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = partials[blockIdx.x] + block_exclusive_scan(s, smem, total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < elements) data[base + k] = run;
        run += v[k];
    }
}

// ------------------------------------------------------------- sort finish

__global__ void __launch_bounds__(kBlock) k_bucket(uint32_t n, const uint32_t *__restrict__ hash,
                                                   const uint32_t *__restrict__ slot,
                                                   const uint32_t *__restrict__ cell_first,
                                                   uint32_t *__restrict__ tmp, const uint32_t *__restrict__ skip) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (skip && *skip)) return;
    tmp[cell_first[hash[i]] + slot[i]] = i;
}

// Stable placement and reorder: the rank of particle i inside its cell is
// the number of bucket-mates with a smaller original index, so the sorted
// order is (hash, original index) -- the order of the reference's stable
// key-value sort seeded with index = i (integration_kernel.cuh:224,
// integration.cu:270-275).  The same thread gathers the particle's data into
// the sorted SoA arrays (reorderDataAndFindCellStartD,
// integration_kernel.cuh:287-295); the cell start/end of the reference are
// the dense offsets cell_first[c], cell_first[c + 1].
__global__ void __launch_bounds__(kBlock) k_rank_reorder(uint32_t n, const uint32_t *__restrict__ hash,
                                                         const uint32_t *__restrict__ cell_first,
                                                         const uint32_t *__restrict__ tmp,
                                                         const float4 *__restrict__ x,
                                                         const int *__restrict__ phase,
                                                         const float *__restrict__ rho0,
                                                         uint32_t *__restrict__ sorted_idx,
                                                         float4 *__restrict__ sorted_x,
                                                         SortedAttr *__restrict__ sorted_attr,
                                                         const uint32_t *__restrict__ skip) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (skip && *skip)) return;
    const uint32_t h = hash[i];
    const uint32_t b = cell_first[h], e = cell_first[h + 1];
    uint32_t rank = 0;
    for (uint32_t k = b; k < e; ++k) rank += (tmp[k] < i) ? 1u : 0u;
    const uint32_t p = b + rank;
    sorted_idx[p] = i;
    sorted_x[p] = x[i];
    SortedAttr a;
    a.phase = phase[i];
    a.rho0 = rho0[i];
    sorted_attr[p] = a;
}

// The whole grid build of a small single-scene system in one block: the
// steps of k_clear_counts / k_hash_count, the scan, k_bucket and
// k_rank_reorder, separated by block barriers instead of launches, with the
// cell counts, hashes, arrival slots and buckets in shared memory (one
// global pass over the particles and the cell offsets).
constexpr int kSmallGridThreads = kScanThreads;
__global__ void __launch_bounds__(kSmallGridThreads) k_grid_small(DevParams P, uint32_t n,
                                                                  const float4 *__restrict__ x,
                                                                  const int *__restrict__ phase,
                                                                  const float *__restrict__ rho0, GridBuffers g) {
    pdl_entry();
    extern __shared__ uint32_t s_small[];
    __shared__ uint32_t smem[32];
    const uint32_t cells = P.num_cells + 1u;
    uint32_t *const cnt = s_small;  // [cells]: counts, then offsets
    uint32_t *const hs = cnt + cells;  // [n] cell of each particle
    uint32_t *const sl = hs + n;       // [n] arrival slot in its cell
    uint32_t *const tmp = sl + n;      // [n] cell-bucketed indices
    for (uint32_t c = threadIdx.x; c < cells; c += blockDim.x) cnt[c] = 0u;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t h = grid_hash(P, grid_pos(P, f3(x[i])));
        hs[i] = h;
        g.hash[i] = h;
        sl[i] = atomicAdd(cnt + h, 1u);
    }
    __syncthreads();
    // exclusive scan, each thread over a contiguous run of cells
    const uint32_t per = (cells + blockDim.x - 1u) / blockDim.x;
    const uint32_t c0 = min(threadIdx.x * per, cells), c1 = min(c0 + per, cells);
    uint32_t sum = 0;
    for (uint32_t c = c0; c < c1; ++c) sum += cnt[c];
    uint32_t total;
    uint32_t run = block_exclusive_scan(sum, smem, total);
    for (uint32_t c = c0; c < c1; ++c) {
        const uint32_t v = cnt[c];
        cnt[c] = run;
        g.cell_first[c] = run;
        run += v;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) tmp[cnt[hs[i]] + sl[i]] = i;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t h = hs[i];
        const uint32_t b = cnt[h], e = cnt[h + 1];
        uint32_t rank = 0;
        for (uint32_t k = b; k < e; ++k) rank += (tmp[k] < i) ? 1u : 0u;
        const uint32_t p = b + rank;
        g.sorted_idx[p] = i;
        g.sorted_x[p] = x[i];
        SortedAttr a;
        a.phase = phase[i];
        a.rho0 = rho0[i];
        g.sorted_attr[p] = a;
    }
}

// Stable in-cell rank only (k_rank_reorder without the data gather).
__global__ void __launch_bounds__(kBlock) k_rank_only(uint32_t n, const uint32_t *__restrict__ hash,
                                                      const uint32_t *__restrict__ cell_first,
                                                      const uint32_t *__restrict__ tmp,
                                                      uint32_t *__restrict__ sorted_idx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hash[i];
    const uint32_t b = cell_first[h], e = cell_first[h + 1];
    uint32_t rank = 0;
    for (uint32_t k = b; k < e; ++k) rank += (tmp[k] < i) ? 1u : 0u;
    sorted_idx[b + rank] = i;
}

// Dense offsets to the reference's cellStart / cellEnd layout
// (integration_kernel.cuh:274-285): empty cells get start 0xffffffff and
// end 0.
__global__ void __launch_bounds__(kBlock) k_cell_ranges(uint32_t cells, const uint32_t *__restrict__ cell_first,
                                                        uint32_t *__restrict__ cell_start,
                                                        uint32_t *__restrict__ cell_end) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const uint32_t b = cell_first[c], e = cell_first[c + 1];
    cell_start[c] = (e > b) ? b : 0xffffffffu;
    cell_end[c] = (e > b) ? e : 0u;
}

__global__ void __launch_bounds__(kBlock) k_refresh_sorted(uint32_t n, const uint32_t *__restrict__ sorted_idx,
                                                           const float4 *__restrict__ x,
                                                           float4 *__restrict__ sorted_x) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sorted_x[i] = x[sorted_idx[i]];
}

// Cell counts cleared (the memset of a grid build), unless *skip.
__global__ void __launch_bounds__(kBlock) k_clear_counts(uint32_t elements, uint32_t *__restrict__ counts,
                                                         const uint32_t *__restrict__ skip) {
    pdl_entry();
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= elements || *skip) return;
    counts[c] = 0u;
}

// Skin-list check: the sorted positions refreshed from x in the sorted
// order of the list's grid, and the largest |x - x_at_build| / h over all
// particles into words[2 + iter] (non-negative floats order like their
// bit patterns, so an integer max).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_skin_check(DevParams P0, uint32_t n, const uint32_t *__restrict__ sidx,
                                                       const float4 *__restrict__ x,
                                                       const float4 *__restrict__ sref,
                                                       float4 *__restrict__ sorted_x, uint32_t *__restrict__ word) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.f;
    if (i < n) {
        const float4 p = x[sidx[i]];
        sorted_x[i] = p;
        const float4 r = sref[i];
        const float dx = p.x - r.x, dy = p.y - r.y, dz = p.z - r.z;
        d = sqrtf(dx * dx + dy * dy + dz * dz) / scene_params<B>(P0, i).h;
        if (!(d <= 3.0e38f)) d = 3.0e38f;  // NaN or inf: never reuse
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0 && d > 0.f) atomicMax(word, __float_as_uint(d));
}

// One thread: reuse the list this iteration iff every particle stayed
// within 0.49 skin h of where it was when the list was built and no list
// overflowed; otherwise clear the overflow mark for the rebuild.
__global__ void k_skin_decide(uint32_t *__restrict__ words, uint32_t iter, float limit) {
    const bool reuse = __uint_as_float(words[2 + iter]) <= limit && words[1] == 0u;
    words[0] = reuse ? 1u : 0u;
    if (!reuse) words[1] = 0u;
    else words[kSkinWords - 1] += 1u;  // reuses in this step
}

// -------------------------------------------------------- group walking

// A group of TPP consecutive lanes of a warp shares one particle: lane l
// takes candidates b + l, b + l + TPP, ... of every stencil range (one
// coalesced TPP x 16-byte load per step), and partial sums meet in xor
// shuffles.  TPP = 1 runs a particle per thread with branch-free inner
// loops.
template <int TPP>
struct Group {
    int lane;       // lane inside the group
    int wl;         // lane inside the warp
    unsigned mask;  // the group's lanes
    __device__ __forceinline__ Group() {
        wl = threadIdx.x & 31;
        lane = wl & (TPP - 1);
        mask = (TPP == 32) ? 0xffffffffu : (((1u << TPP) - 1u) << (wl & ~(TPP - 1)));
    }
    __device__ __forceinline__ float sum(float v) const {
#pragma unroll
        for (int o = TPP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
        return v;
    }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        return (TPP == 1) ? (p ? (1u << wl) : 0u) : (__ballot_sync(mask, p) & mask);
    }
};

__device__ __forceinline__ float sq(float v) { return v * v; }

// Distance from coordinate p to the unwrapped cell k of one axis.
__device__ __forceinline__ float slab_gap(float p, float origin, float cell, int k) {
    const float lo = origin + (float)k * cell;
    return fmaxf(fmaxf(lo - p, p - (lo + cell)), 0.f);
}

// Calls f(b, e) for the sorted-index ranges of the (2 rad + 1)^3 stencil
// around cell g in the reference's order (z outer, y, x inner;
// integration_kernel.cuh:388-398, 549-559); f returns false to stop.
// With trim, stencil rows and cells whose box lies farther than the reach
// from q (1e-4 relative margin) are skipped -- they hold no neighbours, so
// the neighbour sequence, and with it the reference's first-`cap` neighbour
// rule (integration_kernel.cuh:344,508), is unchanged; exact only when no
// two stencil cells alias (DevParams::trim_*).  A row whose kept cells do
// not wrap is one contiguous range of the dense cell offsets; a wrapping
// row goes cell by cell, repeating aliased cells as the reference does.
template <class F>
__device__ __forceinline__ void stencil_ranges(const DevParams &P, float3 q, int3 g, int rad, float reach2,
                                               bool trim, const uint32_t *__restrict__ cell_first, F &&f) {
    const float lim = reach2 * 1.0001f + 1e-30f;
    const float inv_cell = 1.f / P.cell;
    const int zr = stencil_zrad(P, rad);
    for (int dz = -zr; dz <= zr; ++dz) {
        float gz2 = 0.f;
        if (trim && zr == rad) {  // (in 2-D the layer is every particle's, whatever its z)
            const float t = slab_gap(q.z, P.origin.z, P.cell, g.z + dz);
            gz2 = t * t;
            if (gz2 > lim) continue;
        }
        const uint32_t z = (uint32_t)(g.z + dz) & (P.gz - 1u);
        for (int dy = -rad; dy <= rad; ++dy) {
            float gyz2 = gz2;
            if (trim) {
                const float t = slab_gap(q.y, P.origin.y, P.cell, g.y + dy);
                gyz2 += t * t;
                if (gyz2 > lim) continue;
            }
            int xa = -rad, xb = rad;
            if (trim) {
                // cells met by the sphere's slice |x - q.x| <= w, widened
                // by a small margin against rounding
                const float w = sqrtf(lim - gyz2);
                xa = max(xa, __float2int_rd((q.x - w - P.origin.x) * inv_cell - 1e-3f) - g.x);
                xb = min(xb, __float2int_rd((q.x + w - P.origin.x) * inv_cell + 1e-3f) - g.x);
            }
            const uint32_t y = (uint32_t)(g.y + dy) & (P.gy - 1u);
            const uint32_t row = P.cell_base + (z * P.gy + y) * P.gx;
            const int x0 = g.x + xa, x1 = g.x + xb;
            if (x0 >= 0 && x1 < (int)P.gx) {
                if (x0 <= x1 &&
                    !f(__ldg(cell_first + row + (uint32_t)x0), __ldg(cell_first + row + (uint32_t)x1 + 1u)))
                    return;
            } else {
                for (int dx = xa; dx <= xb; ++dx) {
                    const uint32_t c = row + ((uint32_t)(g.x + dx) & (P.gx - 1u));
                    if (!f(__ldg(cell_first + c), __ldg(cell_first + c + 1u))) return;
                }
            }
        }
    }
}

// Group walk with the exact neighbour cap: test(j, q_j, d2) decides this
// lane's candidate; the first `cap` accepted candidates of the group in
// visiting order go to use(j, q_j, d2).  Returns the group's count.
template <int TPP, class Test, class Use>
__device__ __forceinline__ uint32_t group_walk(const DevParams &P, const Group<TPP> &G, float3 q, int3 g,
                                               int rad, float reach2, bool trim,
                                               const float4 *__restrict__ pos,
                                               const uint32_t *__restrict__ cell_first, uint32_t cap,
                                               Test &&test, Use &&use) {
    uint32_t nb = 0;
    stencil_ranges(P, q, g, rad, reach2, trim, cell_first, [&](uint32_t b, uint32_t e) {
        for (uint32_t base = b; base < e; base += TPP) {
            const uint32_t j = base + (uint32_t)G.lane;
            float4 pj = make_float4(0.f, 0.f, 0.f, 0.f);
            float d2 = 0.f;
            bool ok = false;
            if (j < e) {
                pj = pos[j];
                d2 = dist2_exact(q, f3(pj));
                ok = test(j, pj, d2);
            }
            const unsigned m = G.ballot(ok);
            const uint32_t total = (uint32_t)__popc(m);
            if (nb + total >= cap) {
                ok = ok && (uint32_t)__popc(m & ((1u << G.wl) - 1u)) < cap - nb;
                if (ok) use(j, pj, d2);
                nb = cap;
                return false;
            }
            if (ok) use(j, pj, d2);
            nb += total;
        }
        return true;
    });
    return nb;
}

// ----------------------------------------------------------------- lambda

// Per-neighbour terms of findLambdasD (integration_kernel.cuh:561-589),
// evaluated under the neighbour mask `ok` so the candidate loop has no
// data-dependent branch: poly6 weight, and the spiky gradient over rho0
// (zero below the reference's 1e-4 length cut-off).  sw: the neighbour's
// density weight (density_weight), applied to its density term and to the
// particle's own gradient; the pair gradient in the denominator is not
// weighted (the CPU reference's grad(), totalfluidconstraint.cpp:145-158).
struct LambdaAcc {
    float ro, denom;
    float3 grad;
    __device__ __forceinline__ void add(const DevParams &P, bool ok, float d2, float3 dr, float mass_factor,
                                        float spiky_r, float sw = 1.f) {
        const float hm2 = P.h2 - d2;
        ro += ok ? P.poly6 * hm2 * hm2 * hm2 * mass_factor * sw : 0.f;
        const float rs = rsqrtf(fmaxf(d2, kMinSpiky2));
        const float hm = P.h - d2 * rs;
        const float sc = (ok && d2 >= kMinSpiky2) ? spiky_r * hm * hm * rs : 0.f;
        const float3 sg = dr * sc;
        grad -= sg * sw;
        denom += dot3(sg, sg);
    }
};

// The lambda half of GasConstraint::project (cpu/src/constraint/
// gasconstraint.cpp:34-83) for gas particle i (sorted slot), every lane of
// its group taking part: neighbours are the particles with w > 0 (any phase)
// closer than h, first max_nb in visiting order; rho = sum poly6(r) m_j s_j +
// poly6(0) m_i with s_j = gas_solid_w for phases >= CLOTH (S_SOLID, gas
// weights no gradient); grad_j = -spiky(r) / rho0; lambda = -(rho / rho0 -
// 1) / (sum |grad_j|^2 + |sum grad_j|^2 + relaxation).  The gas lambda goes
// to gas.lam (sxl keeps 0, so fluid corrections see no gas lambda, as the
// reference's per-constraint lambdas, gasconstraint.cpp:99), and an open
// gas adds v' (1 - rho / rho0) (-gas_drag) to the particle's force
// (gasconstraint.cpp:80).
template <int TPP>
__device__ void gas_lambda(const DevParams &P, const Group<TPP> &G, uint32_t i, float4 pi4, float rho0,
                           const float4 *__restrict__ sx, const SortedAttr *__restrict__ sattr,
                           const uint32_t *__restrict__ cell_first, const GasBuffers &gas,
                           float4 *__restrict__ sxl) {
    const float3 pi = f3(pi4);
    const float inv_rho0 = 1.f / rho0;
    const float spiky_r = -P.spiky * inv_rho0;
    float ro = 0.f, denom = 0.f;
    float3 grad = make_float3(0.f, 0.f, 0.f);
    group_walk<TPP>(
        P, G, pi, grid_pos(P, pi), P.fluid_rad, P.h2, P.trim_fluid, sx, cell_first, P.max_nb,
        [&](uint32_t j, const float4 &pj, float d2) { return j != i && d2 < P.h2 && pj.w > 0.f; },
        [&](uint32_t j, const float4 &pj, float d2) {
            const float hm2 = P.h2 - d2;
            const float sw = (sattr[j].phase >= kCloth) ? P.gas_solid_w : 1.f;
            ro += P.poly6 * hm2 * hm2 * hm2 / pj.w * sw;
            const float rs = rsqrtf(fmaxf(d2, kMinSpiky2));
            const float hm = P.h - d2 * rs;
            const float sc = (d2 >= kMinSpiky2) ? spiky_r * hm * hm * rs : 0.f;
            const float3 sg = (pi - f3(pj)) * sc;
            grad -= sg;
            denom += dot3(sg, sg);
        });
    ro = G.sum(ro);
    denom = G.sum(denom);
    grad.x = G.sum(grad.x);
    grad.y = G.sum(grad.y);
    grad.z = G.sum(grad.z);
    if (G.lane != 0) return;
    ro += P.poly6_self / pi4.w;
    denom += dot3(grad, grad);
    const float ratio = ro * inv_rho0;
    gas.lam[i] = -(ratio - 1.f) / (denom + P.relax);
    sxl[i] = make_float4(pi.x, pi.y, pi.z, 0.f);
    const uint32_t o = gas.sidx[i];
    if (gas.open[o]) {
        const float4 vv = gas.v[o];
        float4 f = gas.force[o];
        const float k = (1.f - ratio) * -P.gas_drag;
        f.x += vv.x * k;
        f.y += vv.y * k;
        f.z += vv.z * k;
        gas.force[o] = f;
    }
}

// findLambdasD + collideCellRadius (integration_kernel.cuh:481-593): for a
// fluid particle, neighbours are all particles with |r|^2 < h^2 in the
// (2 ceil(h/cell) + 1)^3 stencil (no phase filter), capped at max_nb in
// visiting order.  rho = sum poly6(r) / w_i + poly6(0) / w_i (own inverse
// mass; PBD_FLAG_DENSITY_NEIGHBOR_MASS uses m_j), grad_j = spiky(r) / rho0,
// lambda = -(rho / rho0 - 1) / (sum |grad_j|^2 + |sum grad_j|^2 + eps).
// Non-fluid particles get lambda = 0 (the reference left their slots
// unwritten and read whatever was there, integration_kernel.cuh:636).
// Output: (position, lambda) per sorted slot, the delta pass's one load.
template <int TPP, bool B>
__global__ void __launch_bounds__(kBlock) k_lambda(DevParams P0, uint32_t n, uint32_t iter_left,
                                                   const float4 *__restrict__ sx,
                                                   const SortedAttr *__restrict__ sattr,
                                                   const uint32_t *__restrict__ cell_first,
                                                   float4 *__restrict__ sxl, GasBuffers gas) {
    pdl_entry();
    const Group<TPP> G;
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / TPP;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    if (!scene_active<B>(P, iter_left)) return;
    const SortedAttr a = sattr[i];
    const float4 pi4 = sx[i];
    const float3 pi = f3(pi4);
    if (a.phase == kGas) {
        gas_lambda<TPP>(P, G, i, pi4, a.rho0, sx, sattr, cell_first, gas, sxl);
        return;
    }
    if (a.phase != kFluid) {
        if (G.lane == 0) sxl[i] = make_float4(pi.x, pi.y, pi.z, 0.f);
        return;
    }
    const bool nb_mass = (P.flags & kFlagDensityNeighborMass) != 0u;
    const float inv_w = 1.f / pi4.w;
    const float inv_rho0 = 1.f / a.rho0;
    const float spiky_r = -P.spiky * inv_rho0;  // spiky coefficient over rho0
    const int3 g = grid_pos(P, pi);
    LambdaAcc acc{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
    bool capped = (TPP != 1);
    if (TPP == 1) {
        uint32_t nb = 0;
        stencil_ranges(P, pi, g, P.fluid_rad, P.h2, P.trim_fluid, cell_first, [&](uint32_t b, uint32_t e) {
            for (uint32_t j = b; j < e; ++j) {
                const float4 pj = sx[j];
                const float d2 = dist2_exact(pi, f3(pj));
                const bool ok = d2 < P.h2 && j != i && fluid_nb_ok(P, pj.w);
                nb += ok ? 1u : 0u;
                const float mf = nb_mass ? ((pj.w > 0.f) ? 1.f / pj.w : 0.f) : inv_w;
                acc.add(P, ok, d2, pi - f3(pj), mf, spiky_r, density_weight(P, sattr, j));
            }
            return true;
        });
        if (nb > P.max_nb) {  // only past the neighbour cap: redo with the exact cap
            acc = LambdaAcc{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
            capped = true;
        }
    }
    if (capped) {
        group_walk<TPP>(
            P, G, pi, g, P.fluid_rad, P.h2, P.trim_fluid, sx, cell_first, P.max_nb,
            [&](uint32_t j, const float4 &pj, float d2) { return j != i && d2 < P.h2 && fluid_nb_ok(P, pj.w); },
            [&](uint32_t j, const float4 &pj, float d2) {
                const float mf = nb_mass ? ((pj.w > 0.f) ? 1.f / pj.w : 0.f) : inv_w;
                acc.add(P, true, d2, pi - f3(pj), mf, spiky_r, density_weight(P, sattr, j));
            });
        acc.ro = G.sum(acc.ro);
        acc.denom = G.sum(acc.denom);
        acc.grad.x = G.sum(acc.grad.x);
        acc.grad.y = G.sum(acc.grad.y);
        acc.grad.z = G.sum(acc.grad.z);
    }
    if (G.lane == 0) {
        const float ro = acc.ro + P.poly6_self * inv_w;
        const float denom = acc.denom + dot3(acc.grad, acc.grad);
        sxl[i] = make_float4(pi.x, pi.y, pi.z, -(ro * inv_rho0 - 1.f) / (denom + P.relax));
    }
}

// --------------------------------------------------------- fused particle

__device__ __forceinline__ float scorr_pow(const DevParams &P, float ratio) {
    if (P.scorr_n_int == 4) {
        const float r2 = ratio * ratio;
        return r2 * r2;
    }
    if (P.scorr_n_int > 0) {
        float r = ratio;
        for (int k = 1; k < P.scorr_n_int; ++k) r *= ratio;
        return r;
    }
    return powf(ratio, P.scorr_n);
}

// Per-neighbour term of solveFluidsD (integration_kernel.cuh:615-637):
// (lambda_i + lambda_j + s_corr) * spiky gradient, with the reference's
// (0, EPS, 0) direction below the 1e-4 length cut-off.
__device__ __forceinline__ void delta_add(const DevParams &P, float3 &delta, bool ok, float d2, float3 dr,
                                          float lam_sum, float poly6_ref) {
    const float hm2 = P.h2 - d2;
    const float coef = lam_sum - P.scorr_k * scorr_pow(P, poly6_ref * hm2 * hm2 * hm2);
    const float rs = rsqrtf(fmaxf(d2, kMinSpiky2));
    const float hm = P.h - d2 * rs;
    const bool far = d2 >= kMinSpiky2;
    const float sc = (ok && far) ? coef * -P.spiky * hm * hm * rs : 0.f;
    delta += dr * sc;
    if (ok && !far) {
        const float hz = P.h - sqrtf(d2);
        delta.y += coef * (-P.spiky * hz * hz * kEps);
    }
}

// The delta half of GasConstraint::project (gasconstraint.cpp:86-121) for
// gas particle i, every lane of its group taking part and each returning
// the total: the lambda pass's neighbours (w > 0, closer than h), delta =
// sum (lambda_i + lambda_j + s_corr) spiky(r) / rho0 / (neighbours + 1),
// lambda_j from gas neighbours only, s_corr = -gas_scorr_k (W(r) / W(DQ_P
// h))^n; the spiky gradient is zero below the 1e-4 length cut-off (the
// reference returned zero at r = 0).  The reference's vorticity term goes
// to the force: f += sum (-|w| r_y, |w| r_x, 0) poly6(r) with w = g(r) * v'_j
// componentwise and g the spiky gradient evaluated at |r|^2 in place of
// |r| (gasconstraint.cpp:109-113 passes glm::dot(r, r)), zero for |r|^2 >= h.
// The particle's contact count (gasconstraint.cpp:119) is zero here: gas
// takes no part in contacts.
template <int TPP>
__device__ float3 gas_delta(const DevParams &P, const Group<TPP> &G, uint32_t i, float3 pi, float rho0,
                            const float4 *__restrict__ sx, const SortedAttr *__restrict__ sattr,
                            const uint32_t *__restrict__ cell_first, const GasBuffers &gas) {
    const float lam_i = gas.lam[i];
    float3 delta = make_float3(0.f, 0.f, 0.f), fv = make_float3(0.f, 0.f, 0.f);
    const uint32_t nb = group_walk<TPP>(
        P, G, pi, grid_pos(P, pi), P.fluid_rad, P.h2, P.trim_fluid, sx, cell_first, P.max_nb,
        [&](uint32_t j, const float4 &pj, float d2) { return j != i && d2 < P.h2 && pj.w > 0.f; },
        [&](uint32_t j, const float4 &pj, float d2) {
            const float3 r = pi - f3(pj);
            const float hm2 = P.h2 - d2;
            const float wp = P.poly6 * hm2 * hm2 * hm2;
            const float lam_j = (sattr[j].phase == kGas) ? gas.lam[j] : 0.f;
            const float corr = -P.gas_scorr_k * scorr_pow(P, wp * P.gas_scorr_inv_ref);
            const float rs = rsqrtf(fmaxf(d2, kMinSpiky2));
            const float hm = P.h - d2 * rs;
            const bool far = d2 >= kMinSpiky2;
            const float sc = far ? -P.spiky * hm * hm * rs : 0.f;
            delta += r * ((lam_i + lam_j + corr) * sc);
            if (far && d2 < P.h) {
                const float hq = P.h - d2;
                const float gsc = -P.spiky * hq * hq * rs;
                const float4 vj = gas.v[gas.sidx[j]];
                const float3 w = make_float3(r.x * gsc * vj.x, r.y * gsc * vj.y, r.z * gsc * vj.z);
                const float wl = len3(w) * wp;
                fv.x -= wl * r.y;
                fv.y += wl * r.x;
            }
        });
    delta.x = G.sum(delta.x);
    delta.y = G.sum(delta.y);
    delta.z = G.sum(delta.z);
    fv.x = G.sum(fv.x);
    fv.y = G.sum(fv.y);
    if (G.lane == 0) {
        const uint32_t o = gas.sidx[i];
        float4 f = gas.force[o];
        f.x += fv.x;
        f.y += fv.y;
        gas.force[o] = f;
    }
    return delta / (rho0 * (float)(nb + 1u));
}

// solveFluidsD (integration_kernel.cuh:596-642): same neighbour set as the
// lambda pass; delta = sum (lambda_i + lambda_j + s_corr) spiky(r) with
// s_corr = -k (W(r) / W(dq h))^n; divided by (rho0 + n) (or rho0 with
// PBD_FLAG_DELTA_OVER_RHO0).  Every lane of the group returns the total.
template <int TPP>
__device__ __forceinline__ float3 fluid_delta(const DevParams &P, const Group<TPP> &G, uint32_t i, float3 pi,
                                              float rho0, const float4 *__restrict__ sxl,
                                              const float4 *__restrict__ sx,
                                              const uint32_t *__restrict__ cell_first) {
    const float lam_i = sxl[i].w;
    const float poly6_ref = P.poly6 * P.scorr_inv_ref;
    const int3 g = grid_pos(P, pi);
    float3 delta = make_float3(0.f, 0.f, 0.f);
    uint32_t nb = 0;
    bool capped = (TPP != 1);
    if (TPP == 1) {
        stencil_ranges(P, pi, g, P.fluid_rad, P.h2, P.trim_fluid, cell_first, [&](uint32_t b, uint32_t e) {
            for (uint32_t j = b; j < e; ++j) {
                const float4 pl = sxl[j];
                const float d2 = dist2_exact(pi, f3(pl));
                const bool ok = d2 < P.h2 && j != i && fluid_nb_ok_at(P, sx, j);
                nb += ok ? 1u : 0u;
                if (nb > P.max_nb) return false;  // over the cap: the capped walk below decides
                delta_add(P, delta, ok, d2, pi - f3(pl), lam_i + pl.w, poly6_ref);
            }
            return true;
        });
        if (nb > P.max_nb) {
            delta = make_float3(0.f, 0.f, 0.f);
            capped = true;
        }
    }
    if (capped) {
        nb = group_walk<TPP>(
            P, G, pi, g, P.fluid_rad, P.h2, P.trim_fluid, sxl, cell_first, P.max_nb,
            // (sxl carries lambda in w: the inverse mass comes from sx)
            [&](uint32_t j, const float4 &, float d2) { return j != i && d2 < P.h2 && fluid_nb_ok_at(P, sx, j); },
            [&](uint32_t, const float4 &pl, float d2) {
                delta_add(P, delta, true, d2, pi - f3(pl), lam_i + pl.w, poly6_ref);
            });
        delta.x = G.sum(delta.x);
        delta.y = G.sum(delta.y);
        delta.z = G.sum(delta.z);
    }
    return delta / fluid_delta_div(P, rho0, nb);
}

// v rotated by the unit quaternion q (xyzw).
__device__ __forceinline__ float3 quat_rotate(float4 q, float3 v) {
    const float3 u = make_float3(q.x, q.y, q.z);
    const float3 t = make_float3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x) * 2.f;
    return v + t * q.w + make_float3(u.y * t.z - u.z * t.y, u.z * t.x - u.x * t.z, u.x * t.y - u.y * t.x);
}

// EPSILON of the CPU reference (cpu/src/includes.h:34).
constexpr float kEpsCpu = 0.0001f;

// RigidContactConstraint::project (cpu/src/constraint/
// rigidcontactconstraint.cpp:30-96) for a pair of particles that both carry
// signed-distance data, evaluated for particle `self` (original index) with
// partner `other`; the pair is ordered by original index (the reference's
// i1 < i2, simulation.cpp:171-193), so both particles evaluate the same
// constraint.  Depth and normal come from the particle nearer its surface
// (normal of the first, or minus that of the second); a depth below one
// diameter + EPSILON is replaced by initBoundary (:13-27): the overlap of
// the pair, with the normal reflected against the pair direction when they
// point apart.  The correction d n is shared by the height-scaled inverse
// masses tmass = w e^y (Particle::scaleMass, particle.h:67-73, at the
// start-of-step heights; formed here as the overflow-free shares
// tmass_k / (tmass_1 + tmass_2)) and averaged over the contact count; this
// particle's count stands in for its partner's, as the GPU reference's
// contact friction does.  Friction: the tangential relative displacement
// since the step's start, removed if below sqrt(mu_s mu_s) d (static), else
// cut by min(sqrt(mu_k mu_k) d / |dpt|, 1).
// The correction and friction of RigidContactConstraint::project
// (rigidcontactconstraint.cpp:58-95) for the ordered pair (1, 2) with depth
// d along n, as seen by particle 1 (first) or 2: d n shared by the
// height-scaled inverse masses tmass = w e^y (Particle::scaleMass,
// particle.h:67-73, at the start-of-step heights p.y; formed as the
// overflow-free shares tmass_k / (tmass_1 + tmass_2)) and averaged over
// the contact count cnt (this particle's, for both ends: the Jacobi form
// of the reference's sequential projection, exact when each particle has
// one constraint); then the tangential relative displacement since the
// step's start removed if below sqrt(mu_s mu_s) d (static), else cut by
// min(sqrt(mu_k mu_k) d / |dpt|, 1).  cs, ck: the contact friction
// coefficients.  One compiled copy (not inlined), so that the batched and
// the single-scene solve kernels round its arithmetic alike.
__device__ __noinline__ float3 rigid_contact_apply(float cs, float ck, bool first, float3 x1, float3 x2, float3 p1,
                                                   float3 p2, float w1, float w2, float d, float3 n, float cnt) {
    const float m = fmaxf(p1.y, p2.y);
    const float t1 = w1 * expf(p1.y - m), t2 = w2 * expf(p2.y - m);
    const float tsum = t1 + t2;
    if (!(tsum > 0.f)) return make_float3(0.f, 0.f, 0.f);
    const float a1 = t1 / tsum, a2 = t2 / tsum;
    const float3 dp1 = n * (-a1 * d / cnt), dp2 = n * (a2 * d / cnt);
    float3 out = first ? dp1 : dp2;
    const float3 nf = n * rsqrtf(dot3(n, n));
    // (x1 + dp1 - p1) - (x2 + dp2 - p2), grouped so that the large
    // coordinates cancel before the small corrections are added
    const float3 dpf = ((x1 - p1) - (x2 - p2)) + (dp1 - dp2);
    const float3 dpt = dpf - nf * dot3(dpf, nf);
    const float ldpt = len3(dpt);
    if (ldpt < kEpsCpu) return out;
    const float3 slip = (ldpt < cs * d) ? dpt : dpt * fminf(ck * d / ldpt, 1.f);
    out += first ? slip * -a1 : slip * a2;
    return out;
}

// PBD_FLAG_CPU_CONTACTS, a pair of solid-like particles without
// signed-distance data: RigidContactConstraint::project's plain branch
// (rigidcontactconstraint.cpp:35-41): d = diameter - |x2 - x1| (nothing
// below EPSILON), n = (x2 - x1) / |x2 - x1|, with the pair ordered by
// original index; correction and friction as rigid_contact_apply.
__device__ __forceinline__ float3 cpu_pair_contact(const DevParams &P, uint32_t self, uint32_t other, float3 xs,
                                                   float3 xo, float3 ps, float3 po, float ws, float wo, float cnt) {
    const bool first = self < other;
    const float3 x1 = first ? xs : xo, x2 = first ? xo : xs;
    const float3 x12 = x2 - x1;
    const float len = len3(x12);
    const float d = 2.f * P.r - len;
    if (d < kEpsCpu) return make_float3(0.f, 0.f, 0.f);
    return rigid_contact_apply(P.cs, P.ck, first, x1, x2, first ? ps : po, first ? po : ps, first ? ws : wo,
                               first ? wo : ws, d, x12 / len, cnt);
}

// PBD_FLAG_CPU_CONTACTS, a solid-like particle touching a fluid or gas one:
// ContactConstraint::project (contactconstraint.cpp:13-42) for this
// particle's end: the overlap diameter - |x_s - x_o| shared by the
// height-scaled inverse masses, averaged over the count, no friction (the
// fluid end is not moved here: fluid takes no part in the contact pass, as
// on the reference GPU).
__device__ __forceinline__ float3 cpu_fluid_contact(const DevParams &P, float3 xs, float3 xo, float3 ps, float3 po,
                                                    float ws, float wo, float cnt) {
    const float3 diff = xs - xo;
    const float dist = len3(diff);
    const float mag = dist - 2.f * P.r;
    if (mag > 0.f || dist == 0.f) return make_float3(0.f, 0.f, 0.f);
    const float m = fmaxf(ps.y, po.y);
    const float ts = ws * expf(ps.y - m), to = wo * expf(po.y - m);
    const float tsum = ts + to;
    if (!(tsum > 0.f)) return make_float3(0.f, 0.f, 0.f);
    return diff * (-(ts / tsum) * mag / (dist * cnt));
}

// Walls a particle touches at e (the CPU reference's boundary detection,
// simulation.cpp:202-224: per axis the lower wall, else the upper one).
__device__ __forceinline__ uint32_t cpu_wall_count(const DevParams &P, float3 e) {
    uint32_t k = 0;
    k += (e.x < P.bmin.x + P.r || e.x > P.bmax.x - P.r) ? 1u : 0u;
    k += (e.y < P.bmin.y + P.r || e.y > P.bmax.y - P.r) ? 1u : 0u;
    if (!(P.flags & kFlagTwoD)) k += (e.z < P.bmin.z + P.r || e.z > P.bmax.z - P.r) ? 1u : 0u;
    return k;
}

__device__ __forceinline__ float3 sdf_contact(const DevParams &P, uint32_t self, uint32_t other, float3 xs,
                                              float3 xo, float3 ps, float3 po, float ws, float wo, float ds,
                                              float dso, float3 ns, float3 no, float cnt) {
    const bool first = self < other;
    const float3 x1 = first ? xs : xo, x2 = first ? xo : xs;
    const float3 p1 = first ? ps : po, p2 = first ? po : ps;
    const float w1 = first ? ws : wo, w2 = first ? wo : ws;
    const float dd1 = first ? ds : dso, dd2 = first ? dso : ds;
    float d;
    float3 n;
    if (dd1 < dd2) {
        d = dd1;
        n = first ? ns : no;
    } else {
        d = dd2;
        n = -(first ? no : ns);
    }
    const float diam = 2.f * P.r;
    if (d < diam + kEpsCpu) {
        float3 x12 = x1 - x2;
        const float len = len3(x12);
        d = diam - len;
        if (d < kEpsCpu) return make_float3(0.f, 0.f, 0.f);
        x12 = len > kEpsCpu ? x12 / len : make_float3(0.f, 1.f, 0.f);
        const float dp = dot3(x12, n);
        n = dp < 0.f ? x12 - n * (2.f * dp) : x12;
    }
    return rigid_contact_apply(P.cs, P.ck, first, x1, x2, p1, p2, w1, w2, d, n, cnt);
}

// collideD + collideCell (integration_kernel.cuh:303-462): contacts of a
// non-fluid particle with every particle closer than 2.001 r in the 27-cell
// stencil (same-object pairs skipped, capped at max_nb), each averaged over
// the contact count; solid-solid pairs get static/kinetic friction against
// the start-of-step positions.  The reference scales both inverse masses of
// a solid-solid pair by the same e^y (y of this particle,
// integration_kernel.cuh:403,422-426); the factor cancels in w_i / (w_i + w_j),
// the only way the masses enter, so it is left out -- exact in real
// arithmetic, and free of the FP32 overflow above y ~ 88 where the
// reference's w e^y became inf and the correction inf * 0 = NaN.  Pairs
// with zero total inverse mass or zero separation are skipped (the
// reference produced NaN there).  Two walks: the count, then the
// corrections.  A pair of solid particles that both carry signed-distance
// data takes the CPU reference's rigid contact instead (sdf_contact).
template <int TPP>
__device__ __forceinline__ float3 contact_delta(const DevParams &P, const Group<TPP> &G, uint32_t i, float4 pi4,
                                                int ph, uint32_t orig, const float4 *__restrict__ sx,
                                                const SortedAttr *__restrict__ sattr,
                                                const uint32_t *__restrict__ sidx,
                                                const uint32_t *__restrict__ cell_first,
                                                const float4 *__restrict__ x_old, const RigidSdf &rs,
                                                float &count_out) {
    const float3 pi = f3(pi4);
    const int3 g = grid_pos(P, pi);
    const bool cpu = (P.flags & kFlagCpuContacts) != 0u;
    // the CPU reference's contact test: closer than a diameter - EPSILON,
    // and never between two fixed particles (simulation.cpp:171-184)
    const float cpu_c = 2.f * P.r - kEpsCpu;
    const float reach2 = cpu ? cpu_c * cpu_c : P.collide2;
    auto test = [&](uint32_t j, const float4 &qj, float d2) {
        if (j == i || !(d2 < reach2)) return false;
        if (cpu && pi4.w == 0.f && qj.w == 0.f) return false;
        const int phj = sattr[j].phase;
        return !(ph > kSolid && ph == phj);
    };
    const uint32_t nb = group_walk<TPP>(P, G, pi, g, 1, reach2, P.trim_contact, sx, cell_first, P.max_nb,
                                        test, [](uint32_t, const float4 &, float) {});
    // the CPU reference averages over every constraint of the group:
    // contacts and walls (updateCounts)
    const float fnb = (float)nb + (cpu ? (float)cpu_wall_count(P, pi) : 0.f);
    count_out = fnb;
    float3 delta = make_float3(0.f, 0.f, 0.f);
    if (nb == 0) return delta;
    const float w = pi4.w;
    const float3 prev = f3(x_old[orig]);
    // this particle's signed-distance data, its normal in the world frame
    float4 si = make_float4(0.f, 0.f, 0.f, -1.f);
    float3 ni = make_float3(0.f, 0.f, 0.f);
    if ((P.flags & kFlagHasSdf) && ph >= kSolid) {
        si = rs.sdf[orig];
        if (si.w >= 0.f) ni = quat_rotate(rs.quat[rs.body[orig]], f3(si));
    }
    group_walk<TPP>(P, G, pi, g, 1, reach2, P.trim_contact, sx, cell_first, nb, test,
                    [&](uint32_t j, const float4 &pj4, float) {
        const int phj = sattr[j].phase;
        if (si.w >= 0.f && phj >= kSolid) {
            const uint32_t oj = sidx[j];
            const float4 sj = rs.sdf[oj];
            if (sj.w >= 0.f) {
                delta += sdf_contact(P, orig, oj, pi, f3(pj4), prev, f3(x_old[oj]), w, pj4.w, si.w, sj.w, ni,
                                     quat_rotate(rs.quat[rs.body[oj]], f3(sj)), fnb);
                return;
            }
        }
        if (cpu) {
            const uint32_t oj = sidx[j];
            if (phj >= kCloth) delta += cpu_pair_contact(P, orig, oj, pi, f3(pj4), prev, f3(x_old[oj]), w, pj4.w, fnb);
            else delta += cpu_fluid_contact(P, pi, f3(pj4), prev, f3(x_old[oj]), w, pj4.w, fnb);
            return;
        }
        const float3 pj = f3(pj4);
        const float3 diff = pi - pj;
        const float dist = len3(diff);
        const float mag = dist - P.collide_dist;
        const float colw = w, colw2 = pj4.w;
        const float wsum = colw + colw2;
        if (wsum == 0.f || dist == 0.f) return;
        const float scale = mag / wsum;
        const float3 dp = diff * (scale / dist);
        const float3 dp1 = (-colw * dp) / fnb;
        const float3 dp2 = (colw2 * dp) / fnb;
        delta += dp1;
        if (ph < kSolid || phj < kSolid) return;
        const float3 prev2 = f3(x_old[sidx[j]]);
        const float3 nf = diff * rsqrtf(dot3(diff, diff));
        const float3 dprel = (pi + dp1 - prev) - (prev + dp2 - prev2);
        const float3 dpt = dprel - nf * dot3(dprel, nf);
        const float ldpt = len3(dpt);
        if (ldpt < kEps) return;
        if (ldpt < P.cs * dist) delta -= dpt * colw / wsum;
        else delta -= dpt * fminf(P.ck * dist / ldpt, 1.f);
    });
    delta.x = G.sum(delta.x);
    delta.y = G.sum(delta.y);
    delta.z = G.sum(delta.z);
    return delta;
}

// ------------------------------------------------------- neighbour lists

// Per-iteration neighbour list, one thread per particle: the lambda pass
// walks the stencil once, testing candidates only, and records every
// neighbour's sorted index in visiting order (four to a uint4, slot-major
// so that reading slot q of 32 consecutive particles is one coalesced
// 512-byte load); the per-neighbour arithmetic of lambda, delta and XSPH
// then runs over the list.  The walk itself records row chunks (NbList):
// per run of up to 32 consecutive candidates of a stencil row, its first
// sorted slot and a bit per candidate that is a neighbour (|r| below the
// list radius, any phase, self excluded); lambda's sums step through the
// chunks and store the indices as they go.  Particles whose list does not
// fit (or with more neighbours than the reference's cap) use the exact
// stencil walk instead.

// The lambda pass's count word: neighbours in the low 16 bits, chunks in
// the high 16 (kListNone: no usable list).
constexpr uint32_t kListNone = 0xffff0000u;
__device__ __forceinline__ uint32_t list_nnb(uint32_t c) { return c & 0xffffu; }
__device__ __forceinline__ uint32_t list_nch(uint32_t c) { return c >> 16; }

__device__ __forceinline__ bool list_usable(const DevParams &P, const NbList &L, uint32_t c) {
    return list_nch(c) <= L.chunks && list_nnb(c) <= L.capacity && list_nnb(c) <= P.max_nb;
}

// Steps through a chunk list: next() returns the next neighbour's sorted
// slot, or `self` past the end.  load(q) returns chunk q.
struct ChunkCursor {
    uint32_t b = 0u, m = 0u, q = 0u;
    template <class Load>
    __device__ __forceinline__ uint32_t next(uint32_t nch, uint32_t self, Load &&load) {
        if (m == 0u && q < nch) {
            const uint2 c = load(q++);
            b = c.x;
            m = c.y;
        }
        if (m == 0u) return self;
        const uint32_t k = (uint32_t)__ffs(m) - 1u;
        m &= m - 1u;
        return b + k;
    }
};

// A quad of the index list, read once per pass: PBD_LIST_LOAD 1 keeps it
// out of L1 (which then holds more of the neighbours' gathered values),
// 2 also marks it first for eviction from L2.  Measured on the 1M dam
// break: 514.0 / 518.6 / 520.0 steps/s for 0 / 1 / 2.
#ifndef PBD_LIST_LOAD
#define PBD_LIST_LOAD 2
#endif
__device__ __forceinline__ uint4 ld_list(const uint4 *p) {
    uint4 r;
#if PBD_LIST_LOAD == 2
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p), "l"(pol));
#elif PBD_LIST_LOAD == 1
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p));
#else
    r = __ldg(p);
#endif
    return r;
}

// A quad of the index list written by the lambda pass: PBD_LIST_STORE 1
// marks it first for eviction from L2 (the list is larger than L2; the
// positions the walk reads then stay longer).  Measured on the 1M dam
// break: 520.7 -> 524.9 steps/s.
#ifndef PBD_LIST_STORE
#define PBD_LIST_STORE 1
#endif
__device__ __forceinline__ void st_list(uint4 *p, uint4 v) {
#if PBD_LIST_STORE == 1
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("st.global.L1::no_allocate.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;"
                 :
                 : "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
#else
    *p = v;
#endif
}

// Calls f(j) for the listed neighbours of particle i (count word c).
template <class F>
__device__ __forceinline__ void for_each_listed(const NbList &L, uint32_t i, uint32_t c, F &&f) {
    const uint32_t cnt = min(list_nnb(c), L.capacity);
    for (uint32_t q = 0; 4u * q < cnt; ++q) {
        const uint4 e = ld_list(L.slot + q * L.stride + i);
        const uint32_t left = cnt - 4u * q;
        f(e.x);
        if (left > 1u) f(e.y);
        if (left > 2u) f(e.z);
        if (left > 3u) f(e.w);
    }
}

// Calls f(j, src[j], ok) for the listed neighbours of particle i (count
// word c), a quad at a time: the quad's four gathers are all issued before
// any is used, so their latencies overlap; slots past the end read
// particle i's own entry and come with ok = false (f must then add
// nothing).
template <int QUADS = 1, class T, class F>
__device__ __forceinline__ void gather_listed(const NbList &L, uint32_t i, uint32_t c,
                                              const T *__restrict__ src, F &&f) {
    const uint32_t cnt = min(list_nnb(c), L.capacity);
    for (uint32_t q = 0; 4u * q < cnt; q += QUADS) {
        uint32_t jj[4 * QUADS];
        T v[4 * QUADS];
#pragma unroll
        for (int u = 0; u < QUADS; ++u) {
            const uint32_t qq = q + (uint32_t)u;
            const uint4 e = (4u * qq < cnt) ? ld_list(L.slot + qq * L.stride + i) : make_uint4(i, i, i, i);
            const uint32_t first = 4u * qq;
            jj[4 * u] = first < cnt ? e.x : i;
            jj[4 * u + 1] = first + 1u < cnt ? e.y : i;
            jj[4 * u + 2] = first + 2u < cnt ? e.z : i;
            jj[4 * u + 3] = first + 3u < cnt ? e.w : i;
        }
#pragma unroll
        for (int t = 0; t < 4 * QUADS; ++t) v[t] = src[jj[t]];
#pragma unroll
        for (int t = 0; t < 4 * QUADS; ++t) f(jj[t], v[t], 4u * q + (uint32_t)t < cnt);
    }
}

// The chunks of candidates [b, e) of one stencil row for particle i at pi
// (list radius^2 reach2), in order: emit(chunk) for each chunk holding a
// neighbour.  Returns false when emit does (the list is full).
template <class Emit>
__device__ __forceinline__ bool row_chunks(uint32_t i, float3 pi, float reach2, uint32_t b, uint32_t e,
                                           const float4 *__restrict__ sx, Emit &&emit) {
    for (uint32_t c = b; c < e; c += 32u) {
        const uint32_t len = min(32u, e - c);
        // candidate k shifts in its test bit: the sign of d2 - reach2 is
        // the test d2 < reach2 (the rounded difference keeps the sign of
        // the exact one, and a NaN result is positive on the GPU)
        uint32_t m = 0u;
#pragma unroll kWalkUnroll
        for (uint32_t k = 0; k < len; ++k) {
            const float4 q = __ldg(sx + c + k);
            m = (m << 1) | (__float_as_uint(__fsub_rn(dist2_exact(pi, f3(q)), reach2)) >> 31);
        }
        m = __brev(m) >> (32u - len);            // candidate k at bit k
        if (i - c < len) m &= ~(1u << (i - c));  // not itself
        if (m && !emit(make_uint2(c, m))) return false;
    }
    return true;
}

// Stencil ranges with the radius fixed at compile time (RAD > 0; RAD = 0
// defers to the runtime version).  The per-axis slab gaps are computed once
// and, per z slab, all 2 RAD + 1 row ranges are fetched together, one slab
// ahead of the walk, so their cell-offset loads overlap each other and the
// walk of the slab before.  The x extent of a kept row comes from a reciprocal square
// root (its rounding is covered by the 1e-3-cell widening).  Same visiting
// order and the same exactness conditions as stencil_ranges; a slab with a
// wrapping row is walked row by row, cell by cell where it wraps.
template <int RAD, class F>
__device__ __forceinline__ void stencil_ranges_fixed(const DevParams &P, float3 q, int3 g, int rad, float reach2,
                                                     bool trim, const uint32_t *__restrict__ cell_first, F &&f) {
    if (RAD == 0) {
        stencil_ranges(P, q, g, rad, reach2, trim, cell_first, f);
        return;
    }
    constexpr int W = 2 * RAD + 1;
    const float lim = reach2 * 1.0001f + 1e-30f;
    const float inv_cell = 1.f / P.cell;
    const float qx = (q.x - P.origin.x) * inv_cell;
    float gy2[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const float t = trim ? slab_gap(q.y, P.origin.y, P.cell, g.y + k - RAD) : 0.f;
        gy2[k] = t * t;
    }
    const bool flat = (P.flags & kFlagTwoD) != 0u;  // 2-D: the particles' own z layer only
    const int kz0 = flat ? RAD : 0, kz1 = flat ? RAD + 1 : W;
    // The row ranges of slab kz (empty rows: b = e = 0); true when a kept
    // row wraps in x.
    auto fetch = [&](int kz, uint32_t (&rb)[W], uint32_t (&re)[W]) {
        const float tz = trim && !flat ? slab_gap(q.z, P.origin.z, P.cell, g.z + kz - RAD) : 0.f;
        const float gz2 = tz * tz;
        const uint32_t zrow = ((uint32_t)(g.z + kz - RAD) & (P.gz - 1u)) * P.gy;
        bool wraps = false;
#pragma unroll
        for (int ky = 0; ky < W; ++ky) {
            rb[ky] = re[ky] = 0u;  // empty unless kept
            const float gyz2 = gz2 + gy2[ky];
            if (gz2 <= lim && gyz2 <= lim) {
                int a = -RAD, b = RAD;
                if (trim) {
                    const float r2 = lim - gyz2;
                    const float wc = r2 * rsqrtf(fmaxf(r2, 1e-30f)) * inv_cell;
                    a = max(a, __float2int_rd(qx - wc - 1e-3f) - g.x);
                    b = min(b, __float2int_rd(qx + wc + 1e-3f) - g.x);
                }
                const int x0 = g.x + a, x1 = g.x + b;
                if (x0 >= 0 && x1 < (int)P.gx) {
                    if (x0 <= x1) {
                        const uint32_t row =
                            P.cell_base + (zrow + ((uint32_t)(g.y + ky - RAD) & (P.gy - 1u))) * P.gx;
                        rb[ky] = __ldg(cell_first + row + (uint32_t)x0);
                        re[ky] = __ldg(cell_first + row + (uint32_t)x1 + 1u);
                    }
                } else if (a <= b) {
                    wraps = true;
                }
            }
        }
        return wraps;
    };
    // the next slab's cell-offset loads are issued before this slab is
    // walked, so they arrive during the walk
    uint32_t rb[W], re[W], nb[W], ne[W];
    bool wraps = fetch(kz0, rb, re);
#pragma unroll 1
    for (int kz = kz0; kz < kz1; ++kz) {
        bool nwraps = false;
        if (kz + 1 < kz1) nwraps = fetch(kz + 1, nb, ne);
        if (!wraps) {
#pragma unroll
            for (int ky = 0; ky < W; ++ky)
                if (rb[ky] < re[ky] && !f(rb[ky], re[ky])) return;
        } else {
            // rare: recompute each row (no indexed arrays, which would live
            // in local memory) and walk wrapping rows cell by cell
            const float tz = trim && !flat ? slab_gap(q.z, P.origin.z, P.cell, g.z + kz - RAD) : 0.f;
            const float gz2 = tz * tz;
            const uint32_t zrow = ((uint32_t)(g.z + kz - RAD) & (P.gz - 1u)) * P.gy;
#pragma unroll 1
            for (int ky = 0; ky < W; ++ky) {
                const float gyz2 = gz2 + (trim ? sq(slab_gap(q.y, P.origin.y, P.cell, g.y + ky - RAD)) : 0.f);
                if (gz2 > lim || gyz2 > lim) continue;
                int a = -RAD, b = RAD;
                if (trim) {
                    const float r2 = lim - gyz2;
                    const float wc = r2 * rsqrtf(fmaxf(r2, 1e-30f)) * inv_cell;
                    a = max(a, __float2int_rd(qx - wc - 1e-3f) - g.x);
                    b = min(b, __float2int_rd(qx + wc + 1e-3f) - g.x);
                }
                const uint32_t row = P.cell_base + (zrow + ((uint32_t)(g.y + ky - RAD) & (P.gy - 1u))) * P.gx;
                const int x0 = g.x + a, x1 = g.x + b;
                if (x0 >= 0 && x1 < (int)P.gx) {
                    if (x0 <= x1 && !f(__ldg(cell_first + row + (uint32_t)x0),
                                       __ldg(cell_first + row + (uint32_t)x1 + 1u)))
                        return;
                } else {
                    for (int dx = a; dx <= b; ++dx) {
                        const uint32_t c = row + ((uint32_t)(g.x + dx) & (P.gx - 1u));
                        if (!f(__ldg(cell_first + c), __ldg(cell_first + c + 1u))) return;
                    }
                }
            }
        }
        wraps = nwraps;
#pragma unroll
        for (int ky = 0; ky < W; ++ky) {
            rb[ky] = nb[ky];
            re[ky] = ne[ky];
        }
    }
}

// Stencil radius and trimming of a list build: the list radius is
// (1 + skin) h (h without a skin).
__device__ __forceinline__ int list_rad(const DevParams &P, float skin) {
    if (skin <= 0.f) return P.fluid_rad;
    return (int)ceilf(P.h * (1.f + skin) / P.cell * 1.000001f);
}

// The list build of one fluid particle by its own stencil walk, then
// lambda's sums over the list (add(j, q_j, d2, ok)), which also store its
// indices to the index list.  The walk's first `cols` chunks stay in the
// lane's shared-memory column (chunk q at col[q * CS]); later ones go to
// the global chunk buffer.  A list that does not fit, or passes the
// neighbour cap, takes the exact capped walk instead.  SKIN: the list radius is
// (1 + skin) h, and listed particles farther than h add nothing.  Sets
// L.count[i].
template <int RAD, int CS, bool SKIN, class Add>
__device__ __forceinline__ void lambda_walk_particle(const DevParams &P, const NbList &L, uint32_t i, float3 pi,
                                                     const float4 *__restrict__ sx,
                                                     const uint32_t *__restrict__ cell_first, uint2 *col,
                                                     uint32_t cols, Add &&add) {
    const int3 g = grid_pos(P, pi);
    int rad = P.fluid_rad;
    float reach2 = P.h2;
    // A three-cell stencil is walked whole: the walk is bound by L1 sectors,
    // and lanes of one cell then walk the same rows and load the same
    // candidates together, which saves more sectors than trimming each
    // particle's rows and cells saves candidates.  Wider stencils (cells
    // smaller than h: about one particle per cell) are trimmed.
    bool trim = RAD == 1 ? false : P.trim_fluid && rad > 1;
    if (SKIN) {
        const int r = list_rad(P, L.skin);
        if ((uint32_t)(2 * r + 1) <= min(P.gx, min(P.gy, P.gz))) {
            const float lr = P.h * (1.f + L.skin);
            rad = r;
            reach2 = lr * lr;
            trim = true;
        } else {
            // the skin's stencil would alias on this grid (cells seen
            // twice): a plain list, and no reuse this step
            atomicOr(L.ovf, 1u);
        }
    }
    const uint32_t cap = L.chunks;
    uint32_t nch = 0, nnb = 0;
    bool full = false;
    stencil_ranges_fixed<RAD>(P, pi, g, rad, reach2, trim, cell_first, [&](uint32_t b, uint32_t e) {
        return row_chunks(i, pi, reach2, b, e, sx, [&](uint2 ch) {
            if (nch == cap) {  // does not fit: the rest of the walk does not matter
                full = true;
                return false;
            }
            if (nch < cols) col[nch * (uint32_t)CS] = ch;
            else L.chunk[(size_t)nch * L.stride + i] = ch;
            ++nch;
            nnb += (uint32_t)__popc(ch.y);
            return true;
        });
    });
    const uint32_t c = full ? kListNone : (nch << 16) | nnb;
    L.count[i] = c;
    if (list_usable(P, L, c)) {
        // four gathers in flight before their sums (slots past the end
        // read this particle's own position and add nothing); each four
        // neighbours go to the index list as one uint4
        const float h2 = P.h2;
        ChunkCursor cur;
        auto load = [&](uint32_t q) { return q < cols ? col[q * (uint32_t)CS] : L.chunk[(size_t)q * L.stride + i]; };
        for (uint32_t k = 0; k < nnb; k += 4u) {
            uint32_t jj[4];
            float4 pp[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) jj[t] = cur.next(nch, i, load);
            st_list(L.slot + (k >> 2) * L.stride + i, make_uint4(jj[0], jj[1], jj[2], jj[3]));
#pragma unroll
            for (int t = 0; t < 4; ++t) pp[t] = __ldg(sx + jj[t]);
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float d2 = dist2_exact(pi, f3(pp[t]));
                add(jj[t], pp[t], d2, k + (uint32_t)t < nnb && (!SKIN || d2 < h2));
            }
        }
    } else {
        if (SKIN) atomicOr(L.ovf, 1u);  // this list cannot be reused
        const Group<1> G;
        group_walk<1>(
            P, G, pi, g, P.fluid_rad, P.h2, P.trim_fluid, sx, cell_first, P.max_nb,
            [&](uint32_t j, const float4 &pj, float d2) { return j != i && d2 < P.h2 && fluid_nb_ok(P, pj.w); },
            [&](uint32_t j, const float4 &pj, float d2) { add(j, pj, d2, true); });
    }
}

// findLambdasD (integration_kernel.cuh:481-593) with the list build, one
// lane per particle (lambda_walk_particle; the first `cols` chunks of each
// list in shared memory, col = s_col + lane with stride CS = the block
// size, or none with cols = 0).  SKIN: the list has a skin (build
// positions kept in L.sref), and when it is reused (*L.reuse) there is no
// walk: the old list is filtered at the refreshed positions.  Output as
// k_lambda.
template <int RAD, bool B, bool SKIN, int CS>
__device__ __forceinline__ void lambda_list_body(const DevParams &P0, uint32_t i, uint32_t n, uint32_t iter_left,
                                                 const float4 *__restrict__ sx,
                                                 const SortedAttr *__restrict__ sattr,
                                                 const uint32_t *__restrict__ cell_first,
                                                 float4 *__restrict__ sxl, const NbList &L,
                                                 const GasBuffers &gas, uint2 *col, uint32_t cols) {
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    const bool reuse = SKIN && L.reuse && *L.reuse;
    // A scene sitting out this iteration needs nothing -- except when a skin
    // list is built: every scene's list must exist for the later
    // iterations that reuse it.
    if (!scene_active<B>(P, iter_left) && (reuse || !SKIN)) return;
    const SortedAttr a = sattr[i];
    const float4 pi4 = sx[i];
    const float3 pi = f3(pi4);
    if (SKIN && !reuse) L.sref[i] = pi4;
    if (a.phase == kGas) {  // no list: the gas passes walk the grid (skin lists are off with gas)
        L.count[i] = 0u;
        gas_lambda<1>(P, Group<1>(), i, pi4, a.rho0, sx, sattr, cell_first, gas, sxl);
        return;
    }
    if (a.phase != kFluid) {
        sxl[i] = make_float4(pi.x, pi.y, pi.z, 0.f);
        if (!reuse) L.count[i] = 0u;
        return;
    }
    const float h2 = P.h2;
    const bool nb_mass = (P.flags & kFlagDensityNeighborMass) != 0u;
    const float inv_w = 1.f / pi4.w;
    const float inv_rho0 = 1.f / a.rho0;
    const float spiky_r = -P.spiky * inv_rho0;
    LambdaAcc acc{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
    auto add = [&](uint32_t j, const float4 &pj, float d2, bool ok) {
        const float mf = nb_mass ? ((pj.w > 0.f) ? 1.f / pj.w : 0.f) : inv_w;
        acc.add(P, ok && fluid_nb_ok(P, pj.w), d2, pi - f3(pj), mf, spiky_r, density_weight(P, sattr, j));
    };
    if (reuse) {
        for_each_listed(L, i, L.count[i], [&](uint32_t j) {
            const float4 pj = __ldg(sx + j);
            const float d2 = dist2_exact(pi, f3(pj));
            if (d2 < h2) add(j, pj, d2, true);
        });
    } else {
        lambda_walk_particle<RAD, CS, SKIN>(P, L, i, pi, sx, cell_first, col, cols, add);
    }
    const float ro = acc.ro + P.poly6_self * inv_w;
    const float denom = acc.denom + dot3(acc.grad, acc.grad);
    sxl[i] = make_float4(pi.x, pi.y, pi.z, -(ro * inv_rho0 - 1.f) / (denom + P.relax));
}

// The list build with every chunk stored straight to the global list.
template <int RAD, bool B, bool SKIN>
__global__ void __launch_bounds__(kBlock, 3) k_lambda_list(DevParams P0, uint32_t n, uint32_t iter_left,
                                                        const float4 *__restrict__ sx,
                                                        const SortedAttr *__restrict__ sattr,
                                                        const uint32_t *__restrict__ cell_first,
                                                        float4 *__restrict__ sxl, NbList L, GasBuffers gas) {
    pdl_entry();
    lambda_list_body<RAD, B, SKIN, 1>(P0, blockIdx.x * blockDim.x + threadIdx.x, n, iter_left, sx, sattr,
                                      cell_first, sxl, L, gas, nullptr, 0u);
}

// The list build with each lane's first `cols` chunks in its column of a
// [cols][kListBlock] uint2 array in shared memory (a warp's chunk stores
// are 32 consecutive uint2, free of bank conflicts).
template <int RAD, bool B, bool SKIN>
__global__ void __launch_bounds__(kListBlock, B ? PBD_BATCH_LAMBDA_MIN_BLOCKS : PBD_LAMBDA_MIN_BLOCKS) k_lambda_slist(DevParams P0, uint32_t n, uint32_t iter_left,
                                                                const float4 *__restrict__ sx,
                                                                const SortedAttr *__restrict__ sattr,
                                                                const uint32_t *__restrict__ cell_first,
                                                                float4 *__restrict__ sxl, NbList L,
                                                                GasBuffers gas, uint32_t cols) {
    pdl_entry();
    extern __shared__ uint2 s_col[];
    lambda_list_body<RAD, B, SKIN, kListBlock>(P0, blockIdx.x * kListBlock + threadIdx.x, n, iter_left, sx, sattr,
                                               cell_first, sxl, L, gas, s_col + threadIdx.x, cols);
}

// solveFluidsD (integration_kernel.cuh:596-642) over the lambda pass's list.
__device__ __forceinline__ float3 fluid_delta_list(const DevParams &P, uint32_t i, float3 pi, float rho0,
                                                   const float4 *__restrict__ sxl, const float4 *__restrict__ sx,
                                                   const uint32_t *__restrict__ cell_first, const NbList &L) {
    const uint32_t cnt = L.count[i];
    if (!list_usable(P, L, cnt)) {
        const Group<1> G;
        return fluid_delta<1>(P, G, i, pi, rho0, sxl, sx, cell_first);
    }
    const float lam_i = sxl[i].w;
    const float poly6_ref = P.poly6 * P.scorr_inv_ref;
    const float h2 = P.h2;
    float3 delta = make_float3(0.f, 0.f, 0.f);
    uint32_t nb = 0;
    gather_listed<PBD_DELTA_QUADS>(L, i, cnt, sxl, [&](uint32_t j, const float4 &pl, bool valid) {
        const float d2 = dist2_exact(pi, f3(pl));
        // all of a plain list; a skin list holds more (and a list holds
        // fixed particles, which PBD_FLAG_SKIP_FIXED_NEIGHBORS leaves out)
        const bool ok = valid && d2 < h2 && fluid_nb_ok_at(P, sx, j);
        delta_add(P, delta, ok, d2, pi - f3(pl), lam_i + pl.w, poly6_ref);
        nb += ok ? 1u : 0u;
    });
    return delta / fluid_delta_div(P, rho0, nb);
}

// collide_world_functor (integration_kernel.cuh:57-157): clamp into the box
// shrunk by r with the jitter uniforms, then boundary friction against the
// start-of-step position for phases >= CLOTH.
// PBD_FLAG_CPU_CONTACTS: BoundaryConstraint::project (cpu/src/constraint/
// boundaryconstraint.cpp:14-93) for each wall the particle passed, x then y
// (then z), in turn: back to the wall + r (the reference's extra jitter of
// fluid and gas, frand() * .003, left out), then the tangential part of
// (e - p_old) / count removed if below sqrt(mu_s) r, else cut by
// min(sqrt(mu_k) r / |dpt|, 1).  count: the particle's contacts and walls.
__device__ __forceinline__ float3 cpu_boundaries(const DevParams &P, float3 e, float3 pold, float count) {
    const float r = P.r;
    const int axes = (P.flags & kFlagTwoD) ? 2 : 3;
    if (P.flags & kFlagTwoD) pold.z = P.twod_z;
    for (int a = 0; a < axes; ++a) {
        const float lo = a == 0 ? P.bmin.x : a == 1 ? P.bmin.y : P.bmin.z;
        const float hi = a == 0 ? P.bmax.x : a == 1 ? P.bmax.y : P.bmax.z;
        float v = a == 0 ? e.x : a == 1 ? e.y : e.z;
        float sgn;
        if (v < lo + r) {
            v = lo + r;
            sgn = 1.f;
        } else if (v > hi - r) {
            v = hi - r;
            sgn = -1.f;
        } else {
            continue;
        }
        if (a == 0) e.x = v;
        else if (a == 1) e.y = v;
        else e.z = v;
        const float3 nrm = make_float3(a == 0 ? sgn : 0.f, a == 1 ? sgn : 0.f, a == 2 ? sgn : 0.f);
        const float3 dp = (e - pold) / count;
        const float3 dpt = dp - nrm * dot3(dp, nrm);
        const float ldpt = len3(dpt);
        if (ldpt < kEpsCpu) continue;
        if (ldpt < P.ws * r) e -= dpt;
        else e -= dpt * fminf(P.wk * r / ldpt, 1.f);
    }
    if (P.flags & kFlagTwoD) e.z = P.twod_z;
    return e;
}

__device__ __forceinline__ float3 world_collide(const DevParams &P, float3 e, int phase,
                                                const float4 *__restrict__ x_old, uint32_t orig,
                                                float count = 0.f) {
    if (P.flags & kFlagCpuContacts) {
        if (count < 1.f) count = (float)cpu_wall_count(P, e);
        if (count < 1.f) return (P.flags & kFlagTwoD) ? make_float3(e.x, e.y, P.twod_z) : e;
        return cpu_boundaries(P, e, f3(x_old[orig]), count);
    }
    const float d = P.r;
    float eps = (phase < kSolid) ? d * 0.01f : d * 0.f;
    float3 nrm = make_float3(0.f, 0.f, 0.f);
    const bool twod = (P.flags & kFlagTwoD) != 0u;
    if (e.y < P.bmin.y + P.r) {
        e.y = P.bmin.y + P.r + P.rands[5] * eps;
        nrm.y += 1.f;
    }
    eps = d * 0.01f;
    if (e.x > P.bmax.x - P.r) {
        e.x = P.bmax.x - (P.r + P.rands[0] * eps);
        nrm.x += -1.f;
    }
    if (e.x < P.bmin.x + P.r) {
        e.x = P.bmin.x + (P.r + P.rands[1] * eps);
        nrm.x += 1.f;
    }
    if (e.y > P.bmax.y - P.r) {
        e.y = P.bmax.y - (P.r + P.rands[2] * eps);
        nrm.y += -1.f;
    }
    if (!twod) {
        if (e.z > P.bmax.z - P.r) {
            e.z = P.bmax.z - (P.r + P.rands[3] * eps);
            nrm.z += -1.f;
        }
        if (e.z < P.bmin.z + P.r) {
            e.z = P.bmin.z + (P.r + P.rands[4] * eps);
            nrm.z += 1.f;
        }
    } else {
        e.z = P.twod_z;
    }
    if (len3(nrm) < kEps || phase < kCloth) return e;
    float3 pos = f3(x_old[orig]);
    if (twod) pos.z = P.twod_z;
    const float3 dp = e - pos;
    const float3 dpt = dp - nrm * dot3(dp, nrm);
    const float ldpt = len3(dpt);
    if (ldpt < kEps) return e;
    if (ldpt < P.ws * d) e -= dpt;
    else e -= dpt * fminf(P.wk * d / ldpt, 1.f);
    return e;
}

// One group per sorted particle: the reference's collide, the delta half of
// solveFluids and collideWorld, which touch disjoint particle sets and read
// only the sorted start-of-iteration positions, fused into one pass with one
// write per particle.  mask selects the stages (the stage entry points run
// them one at a time).  NOFLUID leaves the fluid and gas branches out
// (batches without them), which frees registers for a higher occupancy.
constexpr int solve_min_blocks(int tpp, bool batch, bool nofluid) {
    return tpp != 1 ? 0 : nofluid ? PBD_CONTACT_MIN_BLOCKS : batch ? PBD_BATCH_SOLVE_MIN_BLOCKS : PBD_SOLVE_MIN_BLOCKS;
}

template <int TPP, bool B, bool NOFLUID = false>
__global__ void __launch_bounds__(kBlock, solve_min_blocks(TPP, B, NOFLUID)) k_solve(DevParams P0, uint32_t n,
                                                                                  uint32_t mask, uint32_t iter_left,
                                                  const float4 *__restrict__ sx,
                                                  const SortedAttr *__restrict__ sattr,
                                                  const uint32_t *__restrict__ sidx,
                                                  const uint32_t *__restrict__ cell_first,
                                                  const float4 *__restrict__ sxl,
                                                  const float4 *__restrict__ x_old,
                                                  float4 *__restrict__ x, NbList L, bool use_list,
                                                  GasBuffers gas, RigidSdf rs) {
    pdl_entry();
    const Group<TPP> G;
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / TPP;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    if (!scene_active<B>(P, iter_left)) return;
    const SortedAttr a = sattr[i];
    const uint32_t orig = sidx[i];
    const float4 pi4 = sx[i];
    float3 np = f3(pi4);
    bool touched = false;
    float count = 0.f;  // contacts (and, with PBD_FLAG_CPU_CONTACTS, walls) of a contact particle
    if (!NOFLUID && (mask & kDoFluid) && a.phase == kFluid) {
        if constexpr (!NOFLUID) {
            if (TPP == 1 && use_list) np = np + fluid_delta_list(P, i, np, a.rho0, sxl, sx, cell_first, L);
            else np = np + fluid_delta<TPP>(P, G, i, np, a.rho0, sxl, sx, cell_first);
        }
        touched = true;
    } else if (!NOFLUID && (mask & kDoFluid) && a.phase == kGas) {
        if constexpr (!NOFLUID) np = np + gas_delta<TPP>(P, G, i, np, a.rho0, sx, sattr, cell_first, gas);
        touched = true;
    } else if ((mask & kDoContact) && a.phase >= kCloth) {
        np = np + contact_delta<TPP>(P, G, i, pi4, a.phase, orig, sx, sattr, sidx, cell_first, x_old, rs, count);
        touched = true;
    }
    if (G.lane != 0) return;
    if (mask & kDoWorld) {
        if (!touched) np = f3(x[orig]);
        np = world_collide(P, np, a.phase, x_old, orig, count);
        touched = true;
    }
    if (touched) x[orig] = make_float4(np.x, np.y, np.z, pi4.w);
}

// -------------------------------------------------------------- distance

// delta_computing_functor + sort_by_key + reduce_by_key +
// distance_constraint_functor (solver_kernel.cuh:27-72,155-163,
// solver.cu:196-231) as a gather: each constrained particle sums the
// corrections of its incident constraints, d = (x_k - x_o) / |x_k - x_o| *
// (rest - |x_k - x_o|) / 2 (times stiffness), in the order the reference's
// stable sort produced (constraints where k is the first endpoint, then the
// second), and divides by its constraint count.  The reference applied the
// k-th reduced segment to particle k (solver.cu:227-230); here each sum goes
// to its own particle.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_distance_gather(DevParams P0, uint32_t count, uint32_t iter_left,
                                                            const uint32_t *__restrict__ particle,
                                                            const uint32_t *__restrict__ row,
                                                            const uint32_t *__restrict__ other,
                                                            const float *__restrict__ rest,
                                                            const float *__restrict__ stiff,
                                                            const float *__restrict__ occ,
                                                            const float4 *__restrict__ x,
                                                            float4 *__restrict__ out) {
    pdl_entry();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const uint32_t k = particle[s];
    const DevParams P = scene_params<B>(P0, k);
    if (!scene_active<B>(P, iter_left)) return;
    const float4 xk4 = x[k];
    const float3 xk = f3(xk4);
    const bool mass_weighted = (P.flags & kFlagDistanceMassWeighted) != 0u;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    const uint32_t e1 = row[s + 1];
    for (uint32_t e = row[s]; e < e1; ++e) {
        const float4 xo4 = x[other[e]];
        const float3 rel = xk - f3(xo4);
        const float dist = len3(rel);
        if (dist > kMinDistLen) {
            float mag;
            if (mass_weighted) {
                const float ws = xk4.w + xo4.w;
                mag = (ws > 0.f) ? (rest[e] - dist) * (xk4.w / ws) : 0.f;
            } else {
                mag = (rest[e] - dist) * .5f;
            }
            acc += (rel / dist) * (mag * stiff[e]);
        }
    }
    const float o = occ[s];
    out[s] = make_float4(xk.x + acc.x / o, xk.y + acc.y / o, xk.z + acc.z / o, xk4.w);
}

// Writes the gathered positions back and applies pins last
// (point_constraint_functor, solver_kernel.cuh:10-25).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_distance_apply(DevParams P0, uint32_t count, uint32_t iter_left,
                                                           const uint32_t *__restrict__ particle,
                                                           const float4 *__restrict__ tmp,
                                                           const float4 *__restrict__ pin,
                                                           int apply_distance, int apply_pins,
                                                           float4 *__restrict__ x) {
    pdl_entry();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const uint32_t k = particle[s];
    if (!scene_active<B>(scene_params<B>(P0, k), iter_left)) return;
    const bool pinned = apply_pins && pin[s].w != 0.f;
    if (!apply_distance && !pinned) return;
    float4 p = apply_distance ? tmp[s] : x[k];
    if (pinned) {
        const float4 q = pin[s];
        p.x = q.x;
        p.y = q.y;
        p.z = q.z;
    }
    x[k] = p;
}

// ---------------------------------------------------------- shape matching

struct Quat {
    float x, y, z, w;
};

__device__ __forceinline__ void quat_to_mat(const Quat &q, float R[3][3]) {
    const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    R[0][0] = 1.f - 2.f * (yy + zz); R[0][1] = 2.f * (xy - wz);       R[0][2] = 2.f * (xz + wy);
    R[1][0] = 2.f * (xy + wz);       R[1][1] = 1.f - 2.f * (xx + zz); R[1][2] = 2.f * (yz - wx);
    R[2][0] = 2.f * (xz - wy);       R[2][1] = 2.f * (yz + wx);       R[2][2] = 1.f - 2.f * (xx + yy);
}

// Rotation part of A (row-major A[row][col]) by the iterative method of
// Mueller, Bender, Chentanez and Macklin, "A Robust Method to Extract the
// Rotational Part of Deformations" (MIG 2016): starting from q, rotate by
// the axis-angle omega = sum_c (R e_c x A e_c) / (|sum_c R e_c . A e_c| +
// 1e-9) until |omega| vanishes.  Warm-started with the previous rotation, it
// stays well defined for flat or degenerate point sets.
__device__ Quat extract_rotation(const float A[3][3], Quat q, int max_iter) {
    for (int it = 0; it < max_iter; ++it) {
        float R[3][3];
        quat_to_mat(q, R);
        float ox = 0.f, oy = 0.f, oz = 0.f, dsum = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float rx = R[0][c], ry = R[1][c], rz = R[2][c];
            const float ax = A[0][c], ay = A[1][c], az = A[2][c];
            ox += ry * az - rz * ay;
            oy += rz * ax - rx * az;
            oz += rx * ay - ry * ax;
            dsum += rx * ax + ry * ay + rz * az;
        }
        const float inv = 1.f / (fabsf(dsum) + 1.0e-9f);
        ox *= inv;
        oy *= inv;
        oz *= inv;
        const float wlen = sqrtf(ox * ox + oy * oy + oz * oz);
        if (wlen < 1.0e-9f) break;
        const float half = 0.5f * wlen;
        const float sh = sinf(half) / wlen, ch = cosf(half);
        const Quat d = {ox * sh, oy * sh, oz * sh, ch};
        Quat r;  // d * q
        r.w = d.w * q.w - d.x * q.x - d.y * q.y - d.z * q.z;
        r.x = d.w * q.x + d.x * q.w + d.y * q.z - d.z * q.y;
        r.y = d.w * q.y - d.x * q.z + d.y * q.w + d.z * q.x;
        r.z = d.w * q.z + d.x * q.y - d.y * q.x + d.z * q.w;
        const float qn = rsqrtf(r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w);
        q = {r.x * qn, r.y * qn, r.z * qn, r.w * qn};
    }
    return q;
}

constexpr int kShapeIters = 24;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Shape matching (Mueller, Heidelberger, Teschner, Gross 2005): one warp per
// body computes the mass-weighted centre c and A = sum m (x - c) q^T with
// warp-shuffle reductions, extracts R, and moves every particle by
// stiffness * (c + R q - x).  The reference's 2-D counterpart is
// TotalShapeConstraint::project with Body::updateCOM
// (cpu/src/constraint/totalshapeconstraint.cpp:14-24,
// cpu/src/solver/particle.cpp:15-57).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_shapes(DevParams P0, uint32_t iter_left, uint32_t bodies,
                                                   const uint4 *__restrict__ range,
                                                   const float *__restrict__ stiff,
                                                   const float4 *__restrict__ rest,
                                                   float4 *__restrict__ quat,
                                                   float4 *__restrict__ x) {
    pdl_entry();
    const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= bodies) return;
    const uint4 rg = range[b];
    const uint32_t first = rg.x, count = rg.y, roff = rg.z;
    if (!scene_active<B>(scene_params<B>(P0, first), iter_left)) return;
    // centre of mass accumulated relative to the body's first particle, so
    // the FP32 sums carry offsets of the body's size, not of its position
    const float3 o = f3(x[first]);
    float sx = 0.f, sy = 0.f, sz = 0.f, sm = 0.f;
    for (uint32_t k = lane; k < count; k += 32) {
        const float4 p = x[first + k];
        const float m = rest[roff + k].w;
        sx += m * (p.x - o.x);
        sy += m * (p.y - o.y);
        sz += m * (p.z - o.z);
        sm += m;
    }
    sx = warp_sum(sx);
    sy = warp_sum(sy);
    sz = warp_sum(sz);
    sm = warp_sum(sm);
    const float3 c = make_float3(o.x + sx / sm, o.y + sy / sm, o.z + sz / sm);
    float A[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    for (uint32_t k = lane; k < count; k += 32) {
        const float4 p = x[first + k];
        const float4 q = rest[roff + k];
        const float dx = q.w * (p.x - c.x), dy = q.w * (p.y - c.y), dz = q.w * (p.z - c.z);
        A[0][0] += dx * q.x; A[0][1] += dx * q.y; A[0][2] += dx * q.z;
        A[1][0] += dy * q.x; A[1][1] += dy * q.y; A[1][2] += dy * q.z;
        A[2][0] += dz * q.x; A[2][1] += dz * q.y; A[2][2] += dz * q.z;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) A[r][cc] = warp_sum(A[r][cc]);
    float4 q4 = quat[b];
    Quat q = {q4.x, q4.y, q4.z, q4.w};
    q = extract_rotation(A, q, kShapeIters);  // every lane computes the same
    if (lane == 0) quat[b] = make_float4(q.x, q.y, q.z, q.w);
    float R[3][3];
    quat_to_mat(q, R);
    const float st = stiff[b];
    for (uint32_t k = lane; k < count; k += 32) {
        float4 p = x[first + k];
        const float4 r = rest[roff + k];
        // goal minus position formed from small terms: (c - x) + R q
        const float gx = (c.x - p.x) + (R[0][0] * r.x + R[0][1] * r.y + R[0][2] * r.z);
        const float gy = (c.y - p.y) + (R[1][0] * r.x + R[1][1] * r.y + R[1][2] * r.z);
        const float gz = (c.z - p.z) + (R[2][0] * r.x + R[2][1] * r.y + R[2][2] * r.z);
        p.x += gx * st;
        p.y += gy * st;
        p.z += gz * st;
        x[first + k] = p;
    }
}

// --------------------------------------------------------------- velocity

// subtract_functor (integration_kernel.cuh:465-475): v = (x_old - x) / -dt,
// dt = min(dt, max_dt) of the particle's scene.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_velocity(DevParams P0, uint32_t n, float dt,
                                                     const float4 *__restrict__ x,
                                                     const float4 *__restrict__ x_old,
                                                     float4 *__restrict__ v) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = x[i], o = x_old[i];
    const float nd = -fminf(dt, scene_params<B>(P0, i).max_dt);
    v[i] = make_float4((o.x - p.x) / nd, (o.y - p.y) / nd, (o.z - p.z) / nd, 0.f);
}

// ------------------------------------------------------------------- XSPH

// Velocities in sorted order for XSPH, w = the particle's mass as a fluid
// neighbour (1 / w for a fluid particle with w > 0, else 0), so the XSPH
// sum needs no phase lookup.  VEL: the velocity update (k_velocity's
// expression) is done here, for every particle, and written to v as well.
template <bool B, bool VEL>
__global__ void __launch_bounds__(kBlock) k_xsph_gather(DevParams P0, uint32_t n, float dt,
                                                        const uint32_t *__restrict__ sidx,
                                                        const float4 *__restrict__ sx,
                                                        const SortedAttr *__restrict__ sattr,
                                                        const float4 *__restrict__ x,
                                                        const float4 *__restrict__ x_old, float4 *__restrict__ v,
                                                        float4 *__restrict__ vs) {
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = sidx[i];
    float4 vi;
    if constexpr (VEL) {
        const float4 p = x[o], q = x_old[o];
        const float nd = -fminf(dt, scene_params<B>(P0, o).max_dt);
        vi = make_float4((q.x - p.x) / nd, (q.y - p.y) / nd, (q.z - p.z) / nd, 0.f);
        v[o] = vi;
    } else {
        vi = v[o];
    }
    const float w = sx[i].w;
    const float m = (sattr[i].phase == kFluid && w > 0.f) ? 1.f / w : 0.f;
    vs[i] = make_float4(vi.x, vi.y, vi.z, m);
}

// XSPH viscosity (Macklin & Mueller 2013, eq. 17) on fluid particles, made
// dimensionless with the rest density: v_i += c sum_j m_j (v_j - v_i)
// poly6(x_i - x_j) / rho0_i over the fluid neighbours of the last solver
// iteration (the positions its grid was built from), with the step's final
// velocities.
template <int TPP, bool B>
__global__ void __launch_bounds__(kBlock) k_xsph(DevParams P0, uint32_t n, const float4 *__restrict__ sx,
                                                 const SortedAttr *__restrict__ sattr,
                                                 const uint32_t *__restrict__ sidx,
                                                 const uint32_t *__restrict__ cell_first,
                                                 const float4 *__restrict__ vs,
                                                 float4 *__restrict__ v, NbList L, bool use_list) {
    pdl_entry();
    const Group<TPP> G;
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) / TPP;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    if (B && (P.xsph_c == 0.f || P.iterations == 0u)) return;
    const SortedAttr a = sattr[i];
    if (a.phase != kFluid) return;
    const float3 xi = f3(sx[i]);
    const float4 vi4 = vs[i];
    const float3 vi = f3(vi4);
    float3 acc = make_float3(0.f, 0.f, 0.f);
    auto add = [&](uint32_t j, const float4 &xj4, float d2) {
        const float hm2 = P.h2 - d2;
        const float wgt = P.poly6 * hm2 * hm2 * hm2 * ((xj4.w > 0.f) ? 1.f / xj4.w : 0.f);
        acc += (f3(vs[j]) - vi) * wgt;
    };
    bool listed = false;
    if constexpr (TPP == 1) {
        const uint32_t c = use_list ? L.count[i] : 0u;
        listed = use_list && list_usable(P, L, c);
        const uint32_t cnt = listed ? list_nnb(c) : 0u;
        // the last lambda pass listed every neighbour of any phase; a
        // neighbour's fluid mass rides in vs.w (0 for the other phases)
        for (uint32_t q = 0; 4u * q < cnt; ++q) {
            const uint4 e = ld_list(L.slot + q * L.stride + i);
            const uint32_t left = cnt - 4u * q;
            const uint32_t jj[4] = {e.x, left > 1u ? e.y : i, left > 2u ? e.z : i, left > 3u ? e.w : i};
            float4 xx[4], vv[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                xx[t] = sx[jj[t]];
                vv[t] = vs[jj[t]];
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float d2 = dist2_exact(xi, f3(xx[t]));
                const float hm2 = P.h2 - d2;
                const bool ok = (uint32_t)t < left && d2 < P.h2;
                const float wgt = ok ? P.poly6 * hm2 * hm2 * hm2 * vv[t].w : 0.f;
                acc += (f3(vv[t]) - vi) * wgt;
            }
        }
    }
    if (!listed) {
        group_walk<TPP>(
            P, G, xi, grid_pos(P, xi), P.fluid_rad, P.h2, P.trim_fluid, sx, cell_first, P.max_nb,
            [&](uint32_t j, const float4 &, float d2) { return j != i && d2 < P.h2 && sattr[j].phase == kFluid; },
            add);
    }
    acc.x = G.sum(acc.x);
    acc.y = G.sum(acc.y);
    acc.z = G.sum(acc.z);
    if (G.lane != 0) return;
    const float3 nv = vi + acc * (P.xsph_c / a.rho0);
    v[sidx[i]] = make_float4(nv.x, nv.y, nv.z, 0.f);  // w as the velocity update left it
}

// ----------------------------------------------------------- emitters

// The solidification of FluidEmitter::tick (cpu/src/fluidemitter.cpp:14-51)
// over the sorted slots of the last update's grid: a tagged fluid particle
// slower than `speed` at a height <= `height` counts its timer down by 1
// while its lambda of that update is <= 0 (the reference read lambdas[i]
// with i its index in the fluid's particle list, not the particle's own
// index -- here the particle's own lambda), up by dt (to 3) otherwise; at 0
// it becomes a fixed solid at rest (Particle::imass = 0, ph = SOLID, ep = p,
// v = f = 0).  *converted counts the conversions and list[] receives their
// indices (the host pins them there: the GPU step moves w = 0 particles
// like any other in its prediction, integration_kernel.cuh:159-184, and
// holds fixed particles with point constraints, particlesystem.cpp:672-681).
__global__ void __launch_bounds__(kBlock) k_solidify(uint32_t n, float dt, float speed, float height,
                                                     const uint32_t *__restrict__ sidx,
                                                     const float4 *__restrict__ sxl,
                                                     const uint8_t *__restrict__ tag, float *__restrict__ timer,
                                                     float4 *__restrict__ x, float4 *__restrict__ x_old,
                                                     float4 *__restrict__ v, int *__restrict__ phase,
                                                     float4 *__restrict__ force, uint32_t *__restrict__ converted,
                                                     uint32_t *__restrict__ list) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t i = sidx[k];
    if (!tag[i] || phase[i] != kFluid) return;
    const float4 vi = v[i];
    const float4 p = x[i];
    if (!(len3(f3(vi)) < speed && p.y <= height)) return;
    float t = timer[i];
    if (sxl[k].w <= 0.f) {
        t -= 1.f;
        if (t <= 0.f) {
            t = 0.f;
            const float4 fixed = make_float4(p.x, p.y, p.z, 0.f);
            x[i] = fixed;
            x_old[i] = fixed;
            v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            phase[i] = kSolid;
            if (force) force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            list[atomicAdd(converted, 1u)] = i;
        }
    } else {
        t = fminf(t + dt, 3.f);
    }
    timer[i] = t;
}

// The reference's collide wrote each particle as (position, 1) into its
// render buffer (integration_kernel.cuh:461).
__global__ void __launch_bounds__(kBlock) k_vbo(uint32_t n, const float4 *__restrict__ x, float4 *__restrict__ dst) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 p = x[k];
    dst[k] = make_float4(p.x, p.y, p.z, 1.f);
}

__global__ void __launch_bounds__(kBlock) k_finite(uint32_t n, const float4 *__restrict__ x,
                                                   const float4 *__restrict__ v,
                                                   uint32_t *__restrict__ flag) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = x[i], q = v[i];
    const bool ok = isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(q.x) &&
                    isfinite(q.y) && isfinite(q.z);
    if (!ok) atomicOr(flag, 1u);
}

}  // namespace

// ------------------------------------------------------------- launchers

size_t scan_partial_count(uint32_t elements) {
    return (elements + kScanTile - 1) / kScanTile;
}

cudaError_t launch_predict(const DevParams &P, uint32_t n, float dt, float4 *x, float4 *v,
                           float4 *x_old, uint32_t *hash, uint32_t *slot, uint32_t *counts,
                           cudaStream_t s, const GasBuffers &gas) {
    if (n == 0) return cudaSuccess;
    if (P.table) pdl_launch<false>(k_predict<true>, blocks_for(n), kBlock, 0, s, P, n, dt, x, v, x_old, hash, slot, counts, gas);
    else pdl_launch<false>(k_predict<false>, blocks_for(n), kBlock, 0, s, P, n, dt, x, v, x_old, hash, slot, counts, gas);
    return cudaGetLastError();
}

cudaError_t launch_hash_count(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash,
                              uint32_t *slot, uint32_t *counts, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (P.table) pdl_launch(k_hash_count<true>, blocks_for(n), kBlock, 0, s, P, n, x, hash, slot, counts, nullptr);
    else pdl_launch(k_hash_count<false>, blocks_for(n), kBlock, 0, s, P, n, x, hash, slot, counts, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_grid_begin(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash, uint32_t *slot,
                              uint32_t *counts, const uint32_t *skip, cudaStream_t s) {
    const uint32_t elements = P.num_cells + 1u;
    pdl_launch(k_clear_counts, blocks_for(elements), kBlock, 0, s, elements, counts, skip);
    if (n) {
        if (P.table) pdl_launch(k_hash_count<true>, blocks_for(n), kBlock, 0, s, P, n, x, hash, slot, counts, skip);
        else pdl_launch(k_hash_count<false>, blocks_for(n), kBlock, 0, s, P, n, x, hash, slot, counts, skip);
    }
    return cudaGetLastError();
}

cudaError_t launch_skin_check(const DevParams &P, uint32_t n, uint32_t iter, float skin, const GridBuffers &g,
                              const float4 *x, const float4 *sref, uint32_t *words, cudaStream_t s) {
    if (n) {
        if (P.table)
            k_skin_check<true><<<blocks_for(n), kBlock, 0, s>>>(P, n, g.sorted_idx, x, sref, g.sorted_x, words + 2 + iter);
        else
            k_skin_check<false><<<blocks_for(n), kBlock, 0, s>>>(P, n, g.sorted_idx, x, sref, g.sorted_x, words + 2 + iter);
    }
    k_skin_decide<<<1, 1, 0, s>>>(words, iter, 0.49f * skin);
    return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(uint32_t *data, uint32_t elements, uint32_t *partials,
                                  cudaStream_t s, const uint32_t *skip) {
    const uint32_t tiles = (uint32_t)scan_partial_count(elements);
    pdl_launch(k_scan_reduce, tiles, kScanThreads, 0, s, data, elements, partials, skip);
    pdl_launch(k_scan_partials, 1, kScanThreads, 0, s, partials, tiles, skip);
    pdl_launch(k_scan_apply, tiles, kScanThreads, 0, s, data, elements, partials, skip);
    return cudaGetLastError();
}

cudaError_t launch_grid_finish(const DevParams &P, uint32_t n, const GridBuffers &g,
                               const float4 *x, const int *phase, const float *rho0,
                               cudaStream_t s, const uint32_t *skip) {
    cudaError_t e = launch_exclusive_scan(g.cell_first, P.num_cells + 1u, g.scan_part, s, skip);
    if (e != cudaSuccess || n == 0) return e;
    pdl_launch(k_bucket, blocks_for(n), kBlock, 0, s, n, g.hash, g.slot, g.cell_first, g.tmp, skip);
    pdl_launch(k_rank_reorder, blocks_for(n), kBlock, 0, s, n, g.hash, g.cell_first, g.tmp, x, phase, rho0,
                                                    g.sorted_idx, g.sorted_x, g.sorted_attr, skip);
    return cudaGetLastError();
}

size_t small_grid_smem(uint32_t num_cells, uint32_t n) {
    return ((size_t)num_cells + 1u + 3u * (size_t)n) * sizeof(uint32_t);
}

cudaError_t launch_grid_small(const DevParams &P, uint32_t n, const GridBuffers &g, const float4 *x,
                              const int *phase, const float *rho0, cudaStream_t s) {
    const size_t smem = small_grid_smem(P.num_cells, n);
    if (n > kSmallGridN || smem > kSmallGridSmem || P.table) return cudaErrorInvalidValue;
    static bool attr_set = false;  // per process; the attribute holds for every later launch
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_grid_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)kSmallGridSmem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    pdl_launch(k_grid_small, 1u, (unsigned)kSmallGridThreads, smem, s, P, n, x, phase, rho0, g);
    return cudaGetLastError();
}

cudaError_t launch_sort_into_cells(const DevParams &P, uint32_t n, const float4 *x, uint32_t *hash, uint32_t *slot,
                                   uint32_t *cell_first, uint32_t *partials, uint32_t *tmp, uint32_t *sorted_idx,
                                   uint32_t *cell_start, uint32_t *cell_end, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cell_first, 0, ((size_t)P.num_cells + 1u) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    if ((e = launch_hash_count(P, n, x, hash, slot, cell_first, s)) != cudaSuccess) return e;
    if ((e = launch_exclusive_scan(cell_first, P.num_cells + 1u, partials, s)) != cudaSuccess) return e;
    if (n) {
        pdl_launch(k_bucket, blocks_for(n), kBlock, 0, s, n, hash, slot, cell_first, tmp, nullptr);
        k_rank_only<<<blocks_for(n), kBlock, 0, s>>>(n, hash, cell_first, tmp, sorted_idx);
    }
    k_cell_ranges<<<blocks_for(P.num_cells), kBlock, 0, s>>>(P.num_cells, cell_first, cell_start, cell_end);
    return cudaGetLastError();
}

cudaError_t launch_refresh_sorted(uint32_t n, const GridBuffers &g, const float4 *x,
                                  cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_refresh_sorted<<<blocks_for(n), kBlock, 0, s>>>(n, g.sorted_idx, x, g.sorted_x);
    return cudaGetLastError();
}

// Dispatches a kernel template over the supported group sizes (B: batched).
#define PBD_TPP_DISPATCH(tpp, B, KERNEL, ...)                                             \
    switch (tpp) {                                                                        \
    case 1: pdl_launch<false>(KERNEL<1, B>, blocks_for(n * 1u), kBlock, 0, s, __VA_ARGS__); break;      \
    case 2: pdl_launch<false>(KERNEL<2, B>, blocks_for(n * 2u), kBlock, 0, s, __VA_ARGS__); break;      \
    case 4: pdl_launch<false>(KERNEL<4, B>, blocks_for(n * 4u), kBlock, 0, s, __VA_ARGS__); break;      \
    case 8: pdl_launch<false>(KERNEL<8, B>, blocks_for(n * 8u), kBlock, 0, s, __VA_ARGS__); break;      \
    case 16: pdl_launch<false>(KERNEL<16, B>, blocks_for(n * 16u), kBlock, 0, s, __VA_ARGS__); break;   \
    default: pdl_launch<false>(KERNEL<32, B>, blocks_for(n * 32u), kBlock, 0, s, __VA_ARGS__); break;   \
    }

template <bool B>
void lambda_list_dispatch(const DevParams &P, uint32_t n, uint32_t iter_left, const GridBuffers &g, float4 *sxl,
                          const NbList &L, cudaStream_t s, const GasBuffers &gas) {
    const unsigned nb = blocks_for(n);
    // the list radius's stencil; a batch whose fluid scenes differ, and any
    // batch with a skin, runs the runtime-radius walk (rad 0)
    int rad = P.fluid_rad;
    if (L.sref) {
        // (the same single-precision expression as list_rad on the device;
        // the host enables a skin only where its stencil does not alias)
        rad = P.table ? 0 : (int)std::ceil(P.h * (1.f + L.skin) / P.cell * 1.000001f);
    }
    const bool shared = L.assemble == kListShared;
    const unsigned nbs = blocks_for(n, kListBlock);
    const uint32_t cols = std::min(L.chunks, L.sref ? kSharedListColsSkin : kSharedListCols);
    const size_t smem = (size_t)cols * kListBlock * sizeof(uint2);
#define PBD_LIST(R, S)                                                                                      \
    if (shared)                                                                                             \
        pdl_launch<false>(k_lambda_slist<R, B, S>, nbs, kListBlock, smem, s, P, n, iter_left, g.sorted_x, g.sorted_attr,   \
                                                              g.cell_first, sxl, L, gas, cols);             \
    else                                                                                                    \
        pdl_launch<false>(k_lambda_list<R, B, S>, nb, kBlock, 0, s, P, n, iter_left, g.sorted_x, g.sorted_attr, g.cell_first, \
                                                     sxl, L, gas)
    if (L.sref) {
        if (rad == 1) {
            PBD_LIST(1, true);
        } else if (rad == 2) {
            PBD_LIST(2, true);
        } else {
            PBD_LIST(0, true);
        }
    } else {
        if (rad == 1) {
            PBD_LIST(1, false);
        } else if (rad == 2) {
            PBD_LIST(2, false);
        } else {
            PBD_LIST(0, false);
        }
    }
#undef PBD_LIST
}

cudaError_t launch_lambda(const DevParams &P, uint32_t n, uint32_t iter_left, const GridBuffers &g, float4 *sxl,
                          const NbList &L, uint32_t tpp, cudaStream_t s, const GasBuffers &gas) {
    if (n == 0) return cudaSuccess;
    if (tpp == 1 && L.slot) {
        if (P.table) lambda_list_dispatch<true>(P, n, iter_left, g, sxl, L, s, gas);
        else lambda_list_dispatch<false>(P, n, iter_left, g, sxl, L, s, gas);
        return cudaGetLastError();
    }
    if (P.table) {
        PBD_TPP_DISPATCH(tpp, true, k_lambda, P, n, iter_left, g.sorted_x, g.sorted_attr, g.cell_first, sxl, gas);
    } else {
        PBD_TPP_DISPATCH(tpp, false, k_lambda, P, n, iter_left, g.sorted_x, g.sorted_attr, g.cell_first, sxl, gas);
    }
    return cudaGetLastError();
}

cudaError_t launch_solve(const DevParams &P, uint32_t n, uint32_t mask, uint32_t iter_left, const GridBuffers &g,
                         const float4 *sxl, const float4 *x_old, float4 *x, const NbList &L, bool use_list,
                         uint32_t tpp, cudaStream_t s, const GasBuffers &gas, const RigidSdf &sdf) {
    if (n == 0) return cudaSuccess;
    use_list = use_list && L.slot != nullptr;
    if (tpp == 1 && !(mask & kDoFluid)) {
        if (P.table)
            pdl_launch<false>(k_solve<1, true, true>, blocks_for(n), kBlock, 0, s, P, n, mask, iter_left, g.sorted_x, g.sorted_attr,
                                                                     g.sorted_idx, g.cell_first, sxl, x_old, x, L,
                                                                     use_list, gas, sdf);
        else
            pdl_launch<false>(k_solve<1, false, true>, blocks_for(n), kBlock, 0, s, P, n, mask, iter_left, g.sorted_x,
                                                                      g.sorted_attr, g.sorted_idx, g.cell_first, sxl,
                                                                      x_old, x, L, use_list, gas, sdf);
        return cudaGetLastError();
    }
    if (P.table) {
        PBD_TPP_DISPATCH(tpp, true, k_solve, P, n, mask, iter_left, g.sorted_x, g.sorted_attr, g.sorted_idx,
                         g.cell_first, sxl, x_old, x, L, use_list, gas, sdf);
    } else {
        PBD_TPP_DISPATCH(tpp, false, k_solve, P, n, mask, iter_left, g.sorted_x, g.sorted_attr, g.sorted_idx,
                         g.cell_first, sxl, x_old, x, L, use_list, gas, sdf);
    }
    return cudaGetLastError();
}

cudaError_t launch_distance(const DevParams &P, uint32_t iter_left, const ConstraintBuffers &c, float4 *x,
                            bool apply_distance, bool apply_pins, cudaStream_t s) {
    if (c.count == 0) return cudaSuccess;
    apply_distance = apply_distance && c.any_distance;
    apply_pins = apply_pins && c.any_pin;
    if (!apply_distance && !apply_pins) return cudaSuccess;
    const unsigned nb = blocks_for(c.count);
    const int ad = apply_distance ? 1 : 0, ap = apply_pins ? 1 : 0;
    if (P.table) {
        if (apply_distance)
            pdl_launch<false>(k_distance_gather<true>, nb, kBlock, 0, s, P, c.count, iter_left, c.particle, c.row, c.other, c.rest,
                                                          c.stiff, c.occ, x, c.tmp);
        pdl_launch<false>(k_distance_apply<true>, nb, kBlock, 0, s, P, c.count, iter_left, c.particle, c.tmp, c.pin, ad, ap, x);
    } else {
        if (apply_distance)
            pdl_launch<false>(k_distance_gather<false>, nb, kBlock, 0, s, P, c.count, iter_left, c.particle, c.row, c.other, c.rest,
                                                           c.stiff, c.occ, x, c.tmp);
        pdl_launch<false>(k_distance_apply<false>, nb, kBlock, 0, s, P, c.count, iter_left, c.particle, c.tmp, c.pin, ad, ap, x);
    }
    return cudaGetLastError();
}

cudaError_t launch_shapes(const DevParams &P, uint32_t iter_left, const BodyBuffers &b, float4 *x, cudaStream_t s) {
    if (b.count == 0) return cudaSuccess;
    const unsigned nb = blocks_for(b.count * 32u);
    if (P.table) pdl_launch<false>(k_shapes<true>, nb, kBlock, 0, s, P, iter_left, b.count, b.range, b.stiff, b.rest, b.quat, x);
    else pdl_launch<false>(k_shapes<false>, nb, kBlock, 0, s, P, iter_left, b.count, b.range, b.stiff, b.rest, b.quat, x);
    return cudaGetLastError();
}

cudaError_t launch_velocity(const DevParams &P, uint32_t n, float dt, const float4 *x, const float4 *x_old,
                            float4 *v, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (P.table) pdl_launch<false>(k_velocity<true>, blocks_for(n), kBlock, 0, s, P, n, dt, x, x_old, v);
    else pdl_launch<false>(k_velocity<false>, blocks_for(n), kBlock, 0, s, P, n, dt, x, x_old, v);
    return cudaGetLastError();
}

cudaError_t launch_xsph(const DevParams &P, uint32_t n, const GridBuffers &g, float4 *v, float4 *vs,
                        const NbList &L, bool use_list, uint32_t tpp, cudaStream_t s, float dt, const float4 *x,
                        const float4 *x_old) {
    if (n == 0) return cudaSuccess;
    use_list = use_list && L.slot != nullptr;
    const unsigned nb = blocks_for(n);
    if (x && P.table)
        pdl_launch<false>(k_xsph_gather<true, true>, nb, kBlock, 0, s, P, n, dt, g.sorted_idx, g.sorted_x, g.sorted_attr, x, x_old,
                                                         v, vs);
    else if (x)
        pdl_launch<false>(k_xsph_gather<false, true>, nb, kBlock, 0, s, P, n, dt, g.sorted_idx, g.sorted_x, g.sorted_attr, x, x_old,
                                                          v, vs);
    else
        pdl_launch<false>(k_xsph_gather<false, false>, nb, kBlock, 0, s, P, n, dt, g.sorted_idx, g.sorted_x, g.sorted_attr, x,
                                                           x_old, v, vs);
    if (P.table) {
        PBD_TPP_DISPATCH(tpp, true, k_xsph, P, n, g.sorted_x, g.sorted_attr, g.sorted_idx, g.cell_first, vs, v, L,
                         use_list);
    } else {
        PBD_TPP_DISPATCH(tpp, false, k_xsph, P, n, g.sorted_x, g.sorted_attr, g.sorted_idx, g.cell_first, vs, v, L,
                         use_list);
    }
    return cudaGetLastError();
}

cudaError_t launch_solidify(uint32_t n, float dt, float speed, float height, const uint32_t *sidx, const float4 *sxl,
                            const uint8_t *tag, float *timer, float4 *x, float4 *x_old, float4 *v, int *phase,
                            float4 *force, uint32_t *converted, uint32_t *list, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_solidify<<<blocks_for(n), kBlock, 0, s>>>(n, dt, speed, height, sidx, sxl, tag, timer, x, x_old, v, phase,
                                                force, converted, list);
    return cudaGetLastError();
}

cudaError_t launch_vbo(uint32_t n, const float4 *x, float4 *dst, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_vbo<<<blocks_for(n), kBlock, 0, s>>>(n, x, dst);
    return cudaGetLastError();
}

cudaError_t launch_finite_check(uint32_t n, const float4 *x, const float4 *v, uint32_t *flag,
                                cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_finite<<<blocks_for(n), kBlock, 0, s>>>(n, x, v, flag);
    return cudaGetLastError();
}

}  // namespace pbd
