// C ABI of the PBD step: handle lifetime, scene content, the step driver
// (the reference's ParticleSystem::update, gpu/src/particlesystem.cpp:
// 144-246) and the per-stage entry points of gpu/src/cuda/wrappers.cuh.
#include "pbd_system.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

namespace {

thread_local std::string g_create_error;

int fail(pbd_system *s, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (s) s->err = buf;
    else g_create_error = buf;
    return code;
}

#define CUDA_TRY(sys, call)                                                                    \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail((sys), PBD_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

inline bool is_pow2(uint32_t v) { return v && !(v & (v - 1u)); }

int validate_params(const pbd_params *p, std::string &why) {
    if (!p) { why = "params is NULL"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->particle_radius > 0.f)) { why = "particle_radius must be > 0"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->kernel_radius > 0.f)) { why = "kernel_radius must be > 0"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->cell_size > 0.f)) { why = "cell_size must be > 0"; return PBD_ERR_INVALID_ARGUMENT; }
    uint64_t cells = 1;
    for (int k = 0; k < 3; ++k) {
        if (!is_pow2(p->grid_size[k])) { why = "grid_size entries must be powers of two"; return PBD_ERR_INVALID_ARGUMENT; }
        cells *= p->grid_size[k];
    }
    if (cells >= (1ull << 31)) { why = "grid has too many cells (limit 2^31 - 1)"; return PBD_ERR_INVALID_ARGUMENT; }
    if (p->kernel_radius / p->cell_size > 8.f) { why = "kernel_radius / cell_size must be <= 8"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->max_dt > 0.f)) { why = "max_dt must be > 0"; return PBD_ERR_INVALID_ARGUMENT; }
    if (p->max_neighbors == 0) { why = "max_neighbors must be > 0"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->scorr_dq >= 0.f && p->scorr_dq < 1.f)) { why = "scorr_dq must be in [0, 1)"; return PBD_ERR_INVALID_ARGUMENT; }
    if (p->flags & ~PBD_FLAGS_ALL) { why = "unknown bits in flags"; return PBD_ERR_INVALID_ARGUMENT; }
    if ((p->flags & PBD_FLAG_DELTA_OVER_RHO0) && (p->flags & PBD_FLAG_DELTA_OVER_COUNT)) {
        why = "PBD_FLAG_DELTA_OVER_RHO0 and PBD_FLAG_DELTA_OVER_COUNT exclude each other";
        return PBD_ERR_INVALID_ARGUMENT;
    }
    if (!(p->solid_density_weight >= 0.f) || !std::isfinite(p->solid_density_weight)) {
        why = "solid_density_weight must be finite and >= 0";
        return PBD_ERR_INVALID_ARGUMENT;
    }
    if (!(p->gas_scorr_dq >= 0.f && p->gas_scorr_dq < 1.f)) { why = "gas_scorr_dq must be in [0, 1)"; return PBD_ERR_INVALID_ARGUMENT; }
    if (!(p->gas_solid_density_weight >= 0.f) || !std::isfinite(p->gas_solid_density_weight)) {
        why = "gas_solid_density_weight must be finite and >= 0";
        return PBD_ERR_INVALID_ARGUMENT;
    }
    if (!std::isfinite(p->gas_gravity_scale) || !std::isfinite(p->gas_scorr_k) || !std::isfinite(p->gas_drag)) {
        why = "gas_gravity_scale, gas_scorr_k and gas_drag must be finite";
        return PBD_ERR_INVALID_ARGUMENT;
    }
    return PBD_OK;
}

// Derived device constants (the reference's literal coefficients,
// integration_kernel.cuh:25-35, recomputed for any h).
pbd::DevParams make_dev(const pbd_params &p, const float rands[6]) {
    pbd::DevParams d{};
    const double h = p.kernel_radius, pi = 3.14159265358979323846;
    d.gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    d.r = p.particle_radius;
    d.h = p.kernel_radius;
    d.h2 = p.kernel_radius * p.kernel_radius;
    d.cell = p.cell_size;
    d.origin = make_float3(p.world_origin[0], p.world_origin[1], p.world_origin[2]);
    d.gx = p.grid_size[0];
    d.gy = p.grid_size[1];
    d.gz = p.grid_size[2];
    d.num_cells = d.gx * d.gy * d.gz;
    d.bmin = make_float3(p.box_min[0], p.box_min[1], p.box_min[2]);
    d.bmax = make_float3(p.box_max[0], p.box_max[1], p.box_max[2]);
    const double poly6 = 315.0 / (64.0 * pi * std::pow(h, 9.0));
    const double spiky = 45.0 / (pi * std::pow(h, 6.0));
    d.poly6 = (float)poly6;
    d.spiky = (float)spiky;
    d.poly6_self = (float)(poly6 * std::pow(h, 6.0));
    const double dq = p.scorr_dq * h;
    const double t2 = h * h - dq * dq;
    d.scorr_inv_ref = (float)(1.0 / (poly6 * t2 * t2 * t2));
    // kernel-radius units: s_corr enters lambda times h^2, relaxation / h^2
    const bool ku = (p.flags & PBD_FLAG_KERNEL_UNITS) != 0u;
    d.scorr_k = ku ? (float)((double)p.scorr_k * h * h) : p.scorr_k;
    d.scorr_n = p.scorr_n;
    const float rn = std::nearbyint(p.scorr_n);
    d.scorr_n_int = (rn == p.scorr_n && rn >= 1.f && rn <= 16.f) ? (int)rn : 0;
    d.relax = ku ? (float)((double)p.relaxation / (h * h)) : p.relaxation;
    d.xsph_c = p.xsph_c;
    d.cs = p.contact_static_friction;
    d.ck = p.contact_kinetic_friction;
    d.ws = sqrtf(p.wall_static_friction);
    d.wk = sqrtf(p.wall_kinetic_friction);
    d.collide_dist = p.particle_radius * pbd::kCollideScale;
    d.collide2 = d.collide_dist * d.collide_dist;
    d.fluid_rad = (int)std::ceil(p.kernel_radius / p.cell_size);
    // stencils do not alias when every walked axis has room for them (in
    // 2-D the z layer is one, whatever gz)
    const bool twod = (p.flags & PBD_FLAG_TWOD) != 0u;
    const uint32_t gmin = twod ? std::min(d.gx, d.gy) : std::min(d.gx, std::min(d.gy, d.gz));
    d.trim_fluid = (uint32_t)(2 * d.fluid_rad + 1) <= gmin;
    d.trim_contact = 3u <= gmin;
    d.max_nb = p.max_neighbors;
    d.twod_z = p.twod_z;
    {
        // the device's grid_pos expression on the host: IEEE subtract and
        // divide in FP32, then floor
        volatile float t = (p.twod_z - p.world_origin[2]);
        volatile float u = t / p.cell_size;
        d.twod_cz = (int)std::floor((float)u);
    }
    d.flags = p.flags;
    d.solid_w = p.solid_density_weight;
    for (int k = 0; k < 6; ++k) d.rands[k] = rands[k];
    d.gas_gravity = make_float3(p.gravity[0] * p.gas_gravity_scale, p.gravity[1] * p.gas_gravity_scale,
                                p.gravity[2] * p.gas_gravity_scale);
    d.gas_scorr_k = ku ? (float)((double)p.gas_scorr_k * h * h) : p.gas_scorr_k;
    const double gdq = p.gas_scorr_dq * h;
    const double gt2 = h * h - gdq * gdq;
    d.gas_scorr_inv_ref = (float)(1.0 / (poly6 * gt2 * gt2 * gt2));
    d.gas_solid_w = p.gas_solid_density_weight;
    d.gas_drag = p.gas_drag;
    d.iterations = p.iterations;
    d.max_dt = p.max_dt;
    d.cell_base = 0;
    d.table = nullptr;
    d.scene_of = nullptr;
    return d;
}

template <class T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void **)p, count * sizeof(T));
}

template <class T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

void free_constraints(pbd_system *s) {
    dfree(s->cons.particle);
    dfree(s->cons.row);
    dfree(s->cons.other);
    dfree(s->cons.rest);
    dfree(s->cons.stiff);
    dfree(s->cons.occ);
    dfree(s->cons.pin);
    dfree(s->cons.tmp);
    dfree(s->cons.con_a);
    dfree(s->cons.con_b);
    dfree(s->cons.con_rest);
    dfree(s->cons.con_stiff);
    dfree(s->cons.inc_con);
    dfree(s->cons.occ_of);
    s->cons.count = 0;
    s->cons.m = 0;
    s->cons.any_distance = s->cons.any_pin = false;
}

void free_bodies(pbd_system *s) {
    dfree(s->bodies.range);
    dfree(s->bodies.stiff);
    dfree(s->bodies.rest);
    dfree(s->bodies.quat);
    s->bodies.count = 0;
}

void free_grid(pbd_system *s) {
    dfree(s->grid.cell_first);
    dfree(s->grid.scan_part);
    s->grid_cells = 0;
}

void free_list(pbd_system *s) {
    dfree(s->nbl.slot);
    dfree(s->nbl.chunk);
    dfree(s->nbl.count);
    s->nbl.capacity = 0;
    s->nbl.chunks = 0;
    s->list_valid = false;
}

// The neighbour lists of a system with fluid: list_capacity indices per
// particle, and as many row chunks as a quarter of that (a chunk holds a
// neighbour or more).
int alloc_list(pbd_system *s) {
    if (!s->n_fluid || s->nbl.slot || !s->list_capacity) return PBD_OK;
    const uint32_t chunks = s->list_capacity / 4u;
    CUDA_TRY(s, dalloc(&s->nbl.slot, (size_t)(s->list_capacity / 4u) * s->cap));
    CUDA_TRY(s, dalloc(&s->nbl.chunk, (size_t)chunks * s->cap));
    CUDA_TRY(s, dalloc(&s->nbl.count, s->cap));
    s->nbl.capacity = s->list_capacity;
    s->nbl.chunks = chunks;
    s->nbl.stride = s->cap;
    return PBD_OK;
}

// Buffers of the skin-list schedule, once fluid and a skin are both there.
int alloc_skin(pbd_system *s) {
    if (!(s->skin > 0.f) || !s->n_fluid) return PBD_OK;
    if (!s->sref) CUDA_TRY(s, dalloc(&s->sref, s->cap));
    if (!s->skin_words) CUDA_TRY(s, dalloc(&s->skin_words, pbd::kSkinWords));
    return PBD_OK;
}

void drop_graph(pbd_system *s) {
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    s->graph_exec = nullptr;
}

int alloc_grid(pbd_system *s) {
    const uint32_t cells = s->dev.num_cells;
    if (cells == s->grid_cells && s->grid.cell_first) return PBD_OK;
    free_grid(s);
    CUDA_TRY(s, dalloc(&s->grid.cell_first, (size_t)cells + 1u));
    CUDA_TRY(s, dalloc(&s->grid.scan_part, pbd::scan_partial_count(cells + 1u)));
    s->grid_cells = cells;
    s->grid_valid = false;
    return PBD_OK;
}

// Recomputes every scene's parameter block (cells numbered scene after
// scene) and the launch parameters; with several scenes, uploads the scene
// table.  The launch block of a batch carries the total cell count, the
// largest iteration count and the stencil radius shared by every scene with
// fluid (0 when they differ: the kernels then read each scene's own).
int refresh_scenes(pbd_system *s) {
    uint64_t base = 0;
    uint32_t iters = 0;
    int rad = -1;
    for (pbd_scene &sc : s->scenes) {
        sc.dev = make_dev(sc.params, s->rands);
        if (s->n_gas) sc.dev.flags |= pbd::kFlagHasGas;
        if (s->any_sdf) sc.dev.flags |= pbd::kFlagHasSdf;
        sc.dev.cell_base = (uint32_t)base;
        base += sc.dev.num_cells;
        if (base >= (1ull << 31))
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "the scenes' grids hold too many cells in total (limit 2^31 - 1)");
        iters = std::max(iters, sc.params.iterations);
        if (sc.n_fluid) rad = (rad < 0 || rad == sc.dev.fluid_rad) ? sc.dev.fluid_rad : 0;
    }
    if (!s->batched()) {
        s->dev = s->scenes[0].dev;
        return alloc_grid(s);
    }
    const uint32_t S = (uint32_t)s->scenes.size();
    if (S > s->table_cap) {
        dfree(s->d_table);
        const uint32_t want = std::max<uint32_t>(S, 2u * s->table_cap);
        CUDA_TRY(s, dalloc(&s->d_table, want));
        s->table_cap = want;
    }
    std::vector<pbd::DevParams> tab(S);
    for (uint32_t k = 0; k < S; ++k) tab[k] = s->scenes[k].dev;
    CUDA_TRY(s, cudaMemcpy(s->d_table, tab.data(), S * sizeof(pbd::DevParams), cudaMemcpyHostToDevice));
    s->dev = s->scenes[0].dev;
    s->dev.num_cells = (uint32_t)base;
    s->dev.iterations = iters;
    s->dev.fluid_rad = rad < 0 ? 1 : rad;
    s->dev.table = s->d_table;
    s->dev.scene_of = s->d_scene_of;
    return alloc_grid(s);
}

// Scene holding particle slot i.
uint32_t scene_of_slot(const pbd_system *s, uint32_t i) {
    uint32_t lo = 0, hi = (uint32_t)s->scenes.size();
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (s->scenes[mid].first <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

bool any_xsph(const pbd_system *s) {
    for (const pbd_scene &sc : s->scenes)
        if (sc.params.xsph_c != 0.f && sc.n_fluid && sc.params.iterations > 0) return true;
    return false;
}

// Rebuilds the device CSR of distance constraints and pins from the host
// lists.  Per constrained particle the incidences are ordered as the
// reference's stable sort leaves them (first-endpoint occurrences in add
// order, then second-endpoint ones), and occ counts both distance and point
// constraints, as updateOccurences does for each (solver.cu:72-106,122,149).
int upload_constraints(pbd_system *s) {
    free_constraints(s);
    const uint32_t n = s->n;
    std::vector<uint32_t> occ(n, 0), first_cnt(n, 0), second_cnt(n, 0);
    const size_t m = s->dist_a.size();
    for (size_t c = 0; c < m; ++c) {
        ++first_cnt[s->dist_a[c]];
        ++second_cnt[s->dist_b[c]];
        ++occ[s->dist_a[c]];
        ++occ[s->dist_b[c]];
    }
    std::vector<int> pin_of(n, -1);
    for (size_t k = 0; k < s->pin_idx.size(); ++k) {
        ++occ[s->pin_idx[k]];
        pin_of[s->pin_idx[k]] = (int)k;  // the last pin on a particle wins
    }
    std::vector<uint32_t> slot_of(n, UINT32_MAX), particle;
    for (uint32_t k = 0; k < n; ++k)
        if (occ[k]) {
            slot_of[k] = (uint32_t)particle.size();
            particle.push_back(k);
        }
    const uint32_t C = (uint32_t)particle.size();
    if (C == 0) return PBD_OK;
    std::vector<uint32_t> row(C + 1, 0);
    for (uint32_t sidx = 0; sidx < C; ++sidx) {
        const uint32_t k = particle[sidx];
        row[sidx + 1] = row[sidx] + first_cnt[k] + second_cnt[k];
    }
    const uint32_t E = row[C];
    std::vector<uint32_t> other(E), fill_first(C, 0), fill_second(C, 0), inc_con(E);
    std::vector<float> rest(E), stiff(E);
    for (size_t c = 0; c < m; ++c) {
        const uint32_t a = s->dist_a[c], b = s->dist_b[c];
        const uint32_t sa = slot_of[a];
        const uint32_t ea = row[sa] + fill_first[sa]++;
        other[ea] = b;
        rest[ea] = s->dist_rest[c];
        stiff[ea] = s->dist_stiff[c];
        inc_con[ea] = (uint32_t)c;
    }
    for (size_t c = 0; c < m; ++c) {
        const uint32_t a = s->dist_a[c], b = s->dist_b[c];
        const uint32_t sb = slot_of[b];
        const uint32_t eb = row[sb] + first_cnt[b] + fill_second[sb]++;
        other[eb] = a;
        rest[eb] = s->dist_rest[c];
        stiff[eb] = s->dist_stiff[c];
        inc_con[eb] = (uint32_t)c;
    }
    std::vector<float> occf(C);
    std::vector<float4> pin(C, make_float4(0.f, 0.f, 0.f, 0.f));
    for (uint32_t sidx = 0; sidx < C; ++sidx) {
        const uint32_t k = particle[sidx];
        occf[sidx] = (float)occ[k];
        if (pin_of[k] >= 0) {
            const float *pt = &s->pin_pts[3 * (size_t)pin_of[k]];
            pin[sidx] = make_float4(pt[0], pt[1], pt[2], 1.f);
        }
    }
    pbd::ConstraintBuffers &cb = s->cons;
    CUDA_TRY(s, dalloc(&cb.particle, C));
    CUDA_TRY(s, dalloc(&cb.row, C + 1));
    CUDA_TRY(s, dalloc(&cb.other, std::max<uint32_t>(E, 1)));
    CUDA_TRY(s, dalloc(&cb.rest, std::max<uint32_t>(E, 1)));
    CUDA_TRY(s, dalloc(&cb.stiff, std::max<uint32_t>(E, 1)));
    CUDA_TRY(s, dalloc(&cb.occ, C));
    CUDA_TRY(s, dalloc(&cb.pin, C));
    CUDA_TRY(s, dalloc(&cb.tmp, C));
    CUDA_TRY(s, cudaMemcpy(cb.particle, particle.data(), C * 4ull, cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(cb.row, row.data(), (C + 1) * 4ull, cudaMemcpyHostToDevice));
    if (E) {
        CUDA_TRY(s, cudaMemcpy(cb.other, other.data(), E * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.rest, rest.data(), E * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.stiff, stiff.data(), E * 4ull, cudaMemcpyHostToDevice));
    }
    CUDA_TRY(s, cudaMemcpy(cb.occ, occf.data(), C * 4ull, cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(cb.pin, pin.data(), C * sizeof(float4), cudaMemcpyHostToDevice));
    std::vector<float> occ_of(n);
    for (uint32_t k = 0; k < n; ++k) occ_of[k] = (float)occ[k];
    CUDA_TRY(s, dalloc(&cb.occ_of, n));
    CUDA_TRY(s, cudaMemcpy(cb.occ_of, occ_of.data(), n * 4ull, cudaMemcpyHostToDevice));
    if (m) {
        CUDA_TRY(s, dalloc(&cb.con_a, m));
        CUDA_TRY(s, dalloc(&cb.con_b, m));
        CUDA_TRY(s, dalloc(&cb.con_rest, m));
        CUDA_TRY(s, dalloc(&cb.con_stiff, m));
        CUDA_TRY(s, dalloc(&cb.inc_con, E));
        CUDA_TRY(s, cudaMemcpy(cb.con_a, s->dist_a.data(), m * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.con_b, s->dist_b.data(), m * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.con_rest, s->dist_rest.data(), m * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.con_stiff, s->dist_stiff.data(), m * 4ull, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(cb.inc_con, inc_con.data(), E * 4ull, cudaMemcpyHostToDevice));
    }
    cb.m = (uint32_t)m;
    cb.count = C;
    cb.any_distance = m > 0;
    cb.any_pin = !s->pin_idx.empty();
    return PBD_OK;
}

int upload_bodies(pbd_system *s, const std::vector<float4> &quats) {
    free_bodies(s);
    const uint32_t B = (uint32_t)s->body_range.size();
    if (!B) return PBD_OK;
    pbd::BodyBuffers &bb = s->bodies;
    CUDA_TRY(s, dalloc(&bb.range, B));
    CUDA_TRY(s, dalloc(&bb.stiff, B));
    CUDA_TRY(s, dalloc(&bb.rest, s->body_rest.size()));
    CUDA_TRY(s, dalloc(&bb.quat, B));
    CUDA_TRY(s, cudaMemcpy(bb.range, s->body_range.data(), B * sizeof(uint4), cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(bb.stiff, s->body_stiff.data(), B * 4ull, cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(bb.rest, s->body_rest.data(), s->body_rest.size() * sizeof(float4),
                           cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(bb.quat, quats.data(), B * sizeof(float4), cudaMemcpyHostToDevice));
    bb.count = B;
    return PBD_OK;
}

int check_sys(const pbd_system *s) {
    if (!s) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "system handle is NULL");
    return PBD_OK;
}

int use_device(pbd_system *s) {
    CUDA_TRY(s, cudaSetDevice(s->device));
    return PBD_OK;
}

#define SYS_GUARD(s)                          \
    do {                                      \
        if (int rc_ = check_sys(s)) return rc_; \
        if (int rc_ = use_device(s)) return rc_; \
    } while (0)

int need_grid(pbd_system *s) {
    if (!s->grid_valid) return fail(s, PBD_ERR_STATE, "no grid: call pbd_build_grid after the last change of the scene");
    return PBD_OK;
}

// ------------------------------------------------------- stage timing

cudaEvent_t take_event(pbd_system *s) {
    if (!s->event_pool.empty()) {
        cudaEvent_t e = s->event_pool.back();
        s->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

// Brackets one stage group with events when profiling (never inside a
// graph capture) and counts the kernels it launches.
struct Stage {
    pbd_system *s;
    cudaStream_t st;
    int stage;
    uint32_t kernels;
    cudaEvent_t a = nullptr, b = nullptr;
    Stage(pbd_system *s_, cudaStream_t st_, int stage_, uint32_t kernels_)
        : s(s_), st(st_), stage(stage_), kernels(kernels_) {
        if (s->profiling && !s->capturing && kernels) {
            a = take_event(s);
            b = take_event(s);
            if (a && b) cudaEventRecord(a, st);
        }
    }
    ~Stage() {
        s->launches += kernels;
        if (a && b) {
            cudaEventRecord(b, st);
            s->pending.push_back({stage, a, b});
            s->stage_launches[stage] += kernels;
        }
    }
};

int collect_profile(pbd_system *s) {
    for (auto &t : s->pending) {
        CUDA_TRY(s, cudaEventSynchronize(t.stop));
        float ms = 0.f;
        CUDA_TRY(s, cudaEventElapsedTime(&ms, t.start, t.stop));
        s->stage_ms[t.stage] += ms;
        s->event_pool.push_back(t.start);
        s->event_pool.push_back(t.stop);
    }
    s->pending.clear();
    return PBD_OK;
}

// ------------------------------------------------------------- the step

// A single-scene system small enough for the one-block grid build (no
// skin lists: their later iterations use the multi-kernel build).
bool small_grid(const pbd_system *s) {
    return !s->batched() && s->n > 0 && s->n <= pbd::kSmallGridN &&
           pbd::small_grid_smem(s->dev.num_cells, s->n) <= pbd::kSmallGridSmem && s->skin <= 0.f;
}

int build_grid(pbd_system *s, cudaStream_t st, bool hashed_in_predict) {
    const pbd::DevParams &P = s->dev;
    if (small_grid(s)) {  // the prediction did not hash: the block does it all
        Stage t(s, st, PBD_STAGE_GRID, 1u);
        CUDA_TRY(s, pbd::launch_grid_small(P, s->n, s->grid, s->x, s->phase, s->rho0, st));
        s->grid_valid = true;
        s->list_valid = false;
        return PBD_OK;
    }
    Stage t(s, st, PBD_STAGE_GRID, (hashed_in_predict ? 0u : 1u) + 3u + (s->n ? 2u : 0u));
    if (!hashed_in_predict) {
        CUDA_TRY(s, cudaMemsetAsync(s->grid.cell_first, 0, ((size_t)P.num_cells + 1u) * 4u, st));
        CUDA_TRY(s, pbd::launch_hash_count(P, s->n, s->x, s->grid.hash, s->grid.slot, s->grid.cell_first, st));
    }
    CUDA_TRY(s, pbd::launch_grid_finish(P, s->n, s->grid, s->x, s->phase, s->rho0, st));
    s->grid_valid = true;
    s->list_valid = false;
    return PBD_OK;
}

uint32_t solve_mask(const pbd_system *s) {
    uint32_t m = pbd::kDoWorld;
    if (s->any_pbf()) m |= pbd::kDoFluid;
    if (s->n_contact) m |= pbd::kDoContact;
    return m;
}

// The step in the reference's order (particlesystem.cpp:144-246): predict,
// then every iteration rebuilds the grid from the current positions and
// runs contacts + PBF + walls (one fused pass), distance constraints with
// pins, and shape matching; finally the velocity update and XSPH.  With
// several scenes every launch covers all of them; a scene with fewer
// iterations than the batch's most sits out the first ones (its particles
// keep their predicted positions, so the grids it skips change nothing).
// rec (the adjoint's recording, or nullptr): x before the step, then per
// iteration x at its start, after the contact / fluid / wall pass and
// after the distance constraints and pins, then x after the last iteration
// (2 + 3 iterations states of n float4).
int enqueue_update(pbd_system *s, float dt, cudaStream_t st, float4 *rec = nullptr) {
    const pbd::DevParams &P = s->dev;
    const uint32_t n = s->n;
    const size_t nbytes = (size_t)n * sizeof(float4);
    if (rec) CUDA_TRY(s, cudaMemcpyAsync(rec, s->x, nbytes, cudaMemcpyDeviceToDevice, st));
    {
        // predict, with the first grid build's hash and cell counts fused in
        // (not for the one-block grid build, which hashes itself)
        Stage t(s, st, PBD_STAGE_PREDICT, 1);
        const bool small = small_grid(s);
        if (!small) CUDA_TRY(s, cudaMemsetAsync(s->grid.cell_first, 0, ((size_t)P.num_cells + 1u) * 4u, st));
        CUDA_TRY(s, pbd::launch_predict(P, n, dt, s->x, s->v, s->x_old, s->grid.hash, s->grid.slot,
                                        small ? nullptr : s->grid.cell_first, st, s->gas_buffers()));
    }
    const uint32_t mask = solve_mask(s);
    const uint32_t dist_kernels =
        s->cons.count ? (s->cons.any_distance ? 2u : (s->cons.any_pin ? 1u : 0u)) : 0u;
    const uint32_t iters = P.iterations;
    // skin lists: built at the first iteration, reused by later ones while
    // the device check allows (the grid kernels then return at once)
    // (not with gas: the gas passes walk the grid, which a reused list's
    // iterations do not rebuild)
    bool skin = s->skin > 0.f && s->tpp == 1 && s->nbl.slot && s->sref && s->skin_words && s->n_fluid && !s->n_gas &&
                iters > 1;
    if (skin && !P.table) {
        // the skin's stencil must not alias on the grid (a batch checks per
        // scene on the device)
        const int r = (int)std::ceil(P.h * (1.f + s->skin) / P.cell * 1.000001f);
        skin = (uint32_t)(2 * r + 1) <= std::min(P.gx, std::min(P.gy, P.gz));
    }
    pbd::NbList L = s->nbl;
    if (skin) {
        L.skin = s->skin;
        L.sref = s->sref;
        L.ovf = s->skin_words + 1;
        CUDA_TRY(s, cudaMemsetAsync(s->skin_words, 0, pbd::kSkinWords * sizeof(uint32_t), st));
    }
    for (uint32_t it = 0; it < iters; ++it) {
        const uint32_t left = iters - 1u - it;
        if (skin && it > 0 && it + 3u < pbd::kSkinWords) {
            Stage t(s, st, PBD_STAGE_GRID, 2u + 1u + (n ? 6u : 3u));
            CUDA_TRY(s, pbd::launch_skin_check(P, n, it, s->skin, s->grid, s->x, s->sref, s->skin_words, st));
            CUDA_TRY(s, pbd::launch_grid_begin(P, n, s->x, s->grid.hash, s->grid.slot, s->grid.cell_first,
                                               s->skin_words, st));
            CUDA_TRY(s, pbd::launch_grid_finish(P, n, s->grid, s->x, s->phase, s->rho0, st, s->skin_words));
            s->grid_valid = true;
            L.reuse = s->skin_words;
        } else {
            if (int rc = build_grid(s, st, it == 0)) return rc;
            L.reuse = nullptr;
        }
        if (rec) CUDA_TRY(s, cudaMemcpyAsync(rec + (size_t)(1 + 3 * it) * n, s->x, nbytes, cudaMemcpyDeviceToDevice, st));
        if (s->any_pbf()) {
            Stage t(s, st, PBD_STAGE_LAMBDA, 1);
            CUDA_TRY(s, pbd::launch_lambda(P, n, left, s->grid, s->sxl, L, s->tpp, st, s->gas_buffers()));
            s->list_valid = s->tpp == 1 && s->nbl.slot != nullptr;
        }
        {
            Stage t(s, st, PBD_STAGE_SOLVE, 1);
            CUDA_TRY(s, pbd::launch_solve(P, n, mask, left, s->grid, s->sxl, s->x_old, s->x, L,
                                          s->list_valid, s->tpp, st, s->gas_buffers(), s->sdf_buffers()));
        }
        if (rec) CUDA_TRY(s, cudaMemcpyAsync(rec + (size_t)(2 + 3 * it) * n, s->x, nbytes, cudaMemcpyDeviceToDevice, st));
        if (dist_kernels) {
            Stage t(s, st, PBD_STAGE_DISTANCE, dist_kernels);
            CUDA_TRY(s, pbd::launch_distance(P, left, s->cons, s->x, true, true, st));
        }
        if (rec) CUDA_TRY(s, cudaMemcpyAsync(rec + (size_t)(3 + 3 * it) * n, s->x, nbytes, cudaMemcpyDeviceToDevice, st));
        if (s->bodies.count) {
            Stage t(s, st, PBD_STAGE_SHAPES, 1);
            CUDA_TRY(s, pbd::launch_shapes(P, left, s->bodies, s->x, st));
        }
    }
    if (rec) CUDA_TRY(s, cudaMemcpyAsync(rec + (size_t)(1 + 3 * iters) * n, s->x, nbytes, cudaMemcpyDeviceToDevice, st));
    if (any_xsph(s)) {
        // the velocity update is fused into the XSPH gather (its time shows
        // under the XSPH stage)
        Stage t(s, st, PBD_STAGE_XSPH, 2);
        CUDA_TRY(s, pbd::launch_xsph(P, n, s->grid, s->v, s->vs, L, s->list_valid, s->tpp, st, dt, s->x,
                                     s->x_old));
    } else {
        Stage t(s, st, PBD_STAGE_VELOCITY, 1);
        CUDA_TRY(s, pbd::launch_velocity(P, n, dt, s->x, s->x_old, s->v, st));
    }
    ++s->steps;
    return PBD_OK;
}

// One scene: the step is clamped here.  Several: each scene's own clamp is
// applied on the device.
float clamp_dt(const pbd_system *s, float dt) {
    return s->batched() ? dt : std::min(dt, s->scenes[0].params.max_dt);
}

}  // namespace

int pbd_internal_fail(pbd_system *s, int code, const std::string &msg) { return fail(s, code, "%s", msg.c_str()); }
int pbd_internal_guard(pbd_system *s) {
    if (int rc = check_sys(s)) return rc;
    return use_device(s);
}
int pbd_internal_build_grid(pbd_system *s, cudaStream_t st, bool hashed_in_predict) {
    return build_grid(s, st, hashed_in_predict);
}
int pbd_internal_enqueue_update(pbd_system *s, float dt, cudaStream_t st, float4 *rec) {
    return enqueue_update(s, dt, st, rec);
}
bool pbd_internal_any_xsph(const pbd_system *s) { return any_xsph(s); }
float pbd_internal_clamp_dt(const pbd_system *s, float dt) { return clamp_dt(s, dt); }

int pbd_internal_device_params(const pbd_params *params, pbd::DevParams *out, std::string *why) {
    std::string w;
    const int rc = validate_params(params, w);
    if (rc) {
        if (why) *why = w;
        return rc;
    }
    const float zero[6] = {0, 0, 0, 0, 0, 0};
    *out = make_dev(*params, zero);
    return PBD_OK;
}

void pbd_internal_set_thread_error(const std::string &msg) { g_create_error = msg; }

// =================================================================== ABI

extern "C" {

int pbd_abi_version(void) { return PBD_ABI_VERSION; }

void pbd_default_params(pbd_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->particle_radius = 0.25f;
    p->kernel_radius = 2.f;
    p->cell_size = 0.5f;
    p->grid_size[0] = p->grid_size[1] = p->grid_size[2] = 64;
    p->gravity[1] = -9.8f;
    p->box_min[0] = -50.f; p->box_min[1] = 0.f;   p->box_min[2] = -50.f;
    p->box_max[0] = 50.f;  p->box_max[1] = 200.f; p->box_max[2] = 50.f;
    p->iterations = 5;
    p->max_dt = 0.05f;
    p->relaxation = 0.01f;
    p->scorr_k = 0.1f;
    p->scorr_n = 4.f;
    p->scorr_dq = 0.2f;
    p->xsph_c = 0.f;
    p->contact_static_friction = 0.005f;
    p->contact_kinetic_friction = 0.0002f;
    p->wall_static_friction = 0.005f;
    p->wall_kinetic_friction = 0.0002f;
    p->max_neighbors = 500;
    p->twod_z = 0.f;
    p->flags = 0;
    p->solid_density_weight = 1.f;
    p->gas_gravity_scale = -0.2f;
    p->gas_scorr_k = 0.2f;
    p->gas_scorr_dq = 0.25f;
    p->gas_solid_density_weight = 0.5f;
    p->gas_drag = 50.f;
}

const char *pbd_last_error(const pbd_system *s) {
    return s ? s->err.c_str() : g_create_error.c_str();
}

int pbd_create(const pbd_params *params, uint32_t max_particles, pbd_system **out) {
    if (!out) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    std::string why;
    if (validate_params(params, why)) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "%s", why.c_str());
    if (max_particles == 0 || max_particles >= (1u << 31))
        return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "max_particles must be in [1, 2^31)");
    pbd_system *s = new pbd_system();
    s->scenes.emplace_back();
    s->scenes[0].params = *params;
    s->cap = max_particles;
    s->dev = make_dev(*params, s->rands);
    int rc = PBD_OK;
    auto bail = [&](int code) {
        g_create_error = s->err;
        pbd_destroy(s);
        return code;
    };
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        s->err = "no CUDA device";
        return bail(PBD_ERR_CUDA);
    }
    const size_t c = max_particles;
#define ALLOC(ptr, cnt)                                                                       \
    do {                                                                                      \
        cudaError_t e_ = dalloc(&(ptr), (cnt));                                               \
        if (e_ != cudaSuccess) {                                                              \
            s->err = std::string("cudaMalloc failed: ") + cudaGetErrorString(e_);             \
            return bail(PBD_ERR_CUDA);                                                        \
        }                                                                                     \
    } while (0)
    ALLOC(s->x, c);
    ALLOC(s->v, c);
    ALLOC(s->x_old, c);
    ALLOC(s->phase, c);
    ALLOC(s->rho0, c);
    ALLOC(s->sxl, c);
    ALLOC(s->flag, 1);
    ALLOC(s->grid.hash, c);
    ALLOC(s->grid.slot, c);
    ALLOC(s->grid.tmp, c);
    ALLOC(s->grid.sorted_idx, c);
    ALLOC(s->grid.sorted_x, c);
    ALLOC(s->grid.sorted_attr, c);
#undef ALLOC
    if ((rc = refresh_scenes(s))) return bail(rc);
    *out = s;
    return PBD_OK;
}

int pbd_destroy(pbd_system *s) {
    if (!s) return PBD_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    drop_graph(s);
    if (s->graph_stream) cudaStreamDestroy(s->graph_stream);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->copy_fork) cudaEventDestroy(s->copy_fork);
    if (s->copy_join) cudaEventDestroy(s->copy_join);
    for (auto &t : s->pending) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    dfree(s->x);
    dfree(s->v);
    dfree(s->x_old);
    dfree(s->phase);
    dfree(s->rho0);
    dfree(s->sxl);
    free_list(s);
    dfree(s->sref);
    dfree(s->skin_words);
    dfree(s->vs);
    dfree(s->force);
    dfree(s->gas_open);
    dfree(s->glam);
    dfree(s->sdf);
    dfree(s->body_of);
    dfree(s->solid_timer);
    dfree(s->solid_tag);
    dfree(s->solid_count);
    dfree(s->solid_list);
    dfree(s->flag);
    dfree(s->grid.hash);
    dfree(s->grid.slot);
    dfree(s->grid.tmp);
    dfree(s->grid.sorted_idx);
    dfree(s->grid.sorted_x);
    dfree(s->grid.sorted_attr);
    dfree(s->d_table);
    dfree(s->d_scene_of);
    pbd_internal_free_adjoint(s);
    free_grid(s);
    free_constraints(s);
    free_bodies(s);
    delete s;
    return PBD_OK;
}

int pbd_set_params(pbd_system *s, const pbd_params *params) {
    SYS_GUARD(s);
    std::string why;
    if (validate_params(params, why)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "%s", why.c_str());
    const pbd_params old = s->scenes[0].params;
    s->scenes[0].params = *params;
    if (int rc = refresh_scenes(s)) {
        s->scenes[0].params = old;
        refresh_scenes(s);
        return rc;
    }
    s->grid_valid = false;
    s->list_valid = false;
    ++s->version;
    return PBD_OK;
}

int pbd_get_params(const pbd_system *s, pbd_params *out) {
    if (!s || !out) return PBD_ERR_INVALID_ARGUMENT;
    *out = s->scenes[0].params;
    return PBD_OK;
}

int pbd_begin_scene(pbd_system *s, const pbd_params *params, uint32_t *scene_index) {
    SYS_GUARD(s);
    std::string why;
    if (validate_params(params, why)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "%s", why.c_str());
    if (s->scenes.size() >= PBD_MAX_SCENES)
        return fail(s, PBD_ERR_CAPACITY, "a system holds at most %u scenes", (unsigned)PBD_MAX_SCENES);
    if (!s->d_scene_of) {
        CUDA_TRY(s, dalloc(&s->d_scene_of, s->cap));
        CUDA_TRY(s, cudaMemset(s->d_scene_of, 0, (size_t)s->cap * sizeof(uint16_t)));  // all in scene 0
    }
    pbd_scene sc;
    sc.params = *params;
    sc.first = s->n;
    s->scenes.push_back(sc);
    if (int rc = refresh_scenes(s)) {
        s->scenes.pop_back();
        refresh_scenes(s);
        return rc;
    }
    s->grid_valid = false;
    s->list_valid = false;
    ++s->version;
    if (scene_index) *scene_index = (uint32_t)s->scenes.size() - 1u;
    return PBD_OK;
}

uint32_t pbd_num_scenes(const pbd_system *s) { return s ? (uint32_t)s->scenes.size() : 0u; }

int pbd_batch_create(uint32_t n_scenes, const pbd_params *params, const uint32_t *counts, const float *pos_w,
                     const float *vel, const int32_t *phase, const float *rest_density, uint32_t max_particles,
                     pbd_system **out) {
    if (!out) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_scenes == 0 || n_scenes > PBD_MAX_SCENES || !params || !counts)
        return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "n_scenes must be in [1, %u] with params and counts",
                    (unsigned)PBD_MAX_SCENES);
    uint64_t total = 0;
    for (uint32_t k = 0; k < n_scenes; ++k) total += counts[k];
    if (total && !pos_w) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "pos_w is NULL");
    if (total > 0xffffffffull || (max_particles && max_particles < total))
        return fail(nullptr, PBD_ERR_CAPACITY, "the scenes hold %llu particles, capacity %u",
                    (unsigned long long)total, max_particles);
    pbd_system *s = nullptr;
    if (int rc = pbd_create(&params[0], max_particles ? max_particles : (uint32_t)total, &s)) return rc;
    uint64_t off = 0;
    std::vector<int32_t> fluid;
    for (uint32_t k = 0; k < n_scenes; ++k) {
        int rc = k ? pbd_begin_scene(s, &params[k], nullptr) : PBD_OK;
        if (!phase && fluid.size() < counts[k]) fluid.assign(counts[k], PBD_PHASE_FLUID);
        if (!rc && counts[k])
            rc = pbd_add_particles(s, counts[k], pos_w + 4 * off, vel ? vel + 4 * off : nullptr,
                                   phase ? phase + off : fluid.data(), rest_density ? rest_density + off : nullptr,
                                   nullptr);
        if (rc) {
            pbd_internal_set_thread_error(s->err);
            pbd_destroy(s);
            return rc;
        }
        off += counts[k];
    }
    *out = s;
    return PBD_OK;
}

int pbd_get_scene(const pbd_system *s, uint32_t scene, uint32_t *first, uint32_t *count, pbd_params *params) {
    if (!s) return fail(nullptr, PBD_ERR_INVALID_ARGUMENT, "system handle is NULL");
    if (scene >= s->scenes.size()) return PBD_ERR_INVALID_ARGUMENT;
    const pbd_scene &sc = s->scenes[scene];
    if (first) *first = sc.first;
    if (count) *count = sc.count;
    if (params) *params = sc.params;
    return PBD_OK;
}

int pbd_set_scene_params(pbd_system *s, uint32_t scene, const pbd_params *params) {
    SYS_GUARD(s);
    if (scene >= s->scenes.size()) return fail(s, PBD_ERR_INVALID_ARGUMENT, "no scene %u", scene);
    std::string why;
    if (validate_params(params, why)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "%s", why.c_str());
    const pbd_params old = s->scenes[scene].params;
    s->scenes[scene].params = *params;
    if (int rc = refresh_scenes(s)) {
        s->scenes[scene].params = old;
        refresh_scenes(s);
        return rc;
    }
    s->grid_valid = false;
    s->list_valid = false;
    ++s->version;
    return PBD_OK;
}

uint32_t pbd_num_particles(const pbd_system *s) { return s ? s->n : 0u; }
uint32_t pbd_capacity(const pbd_system *s) { return s ? s->cap : 0u; }
uint32_t pbd_num_cells(const pbd_system *s) { return s ? s->dev.num_cells : 0u; }

int pbd_set_wall_jitter(pbd_system *s, const float rands[6]) {
    if (int rc = check_sys(s)) return rc;
    if (!rands) return fail(s, PBD_ERR_INVALID_ARGUMENT, "rands is NULL");
    for (int k = 0; k < 6; ++k) {
        if (!std::isfinite(rands[k])) return fail(s, PBD_ERR_INVALID_ARGUMENT, "rands must be finite");
        s->rands[k] = rands[k];
    }
    if (int rc = refresh_scenes(s)) return rc;
    ++s->version;
    return PBD_OK;
}

int pbd_add_particles(pbd_system *s, uint32_t n, const float *pos_w, const float *vel,
                      const int32_t *phase, const float *rest_density, uint32_t *first_index) {
    SYS_GUARD(s);
    if (n == 0) {
        if (first_index) *first_index = s->n;
        return PBD_OK;
    }
    if (!pos_w || !phase) return fail(s, PBD_ERR_INVALID_ARGUMENT, "pos_w and phase are required");
    if ((uint64_t)s->n + n > s->cap)
        return fail(s, PBD_ERR_CAPACITY, "adding %u particles to %u exceeds capacity %u", n, s->n, s->cap);
    uint32_t nf = 0, nc = 0, ng = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const float *p = pos_w + 4ull * i;
        for (int k = 0; k < 4; ++k)
            if (!std::isfinite(p[k])) return fail(s, PBD_ERR_INVALID_ARGUMENT, "particle %u has a non-finite position/mass", i);
        if (p[3] < 0.f) return fail(s, PBD_ERR_INVALID_ARGUMENT, "particle %u has negative inverse mass", i);
        if (phase[i] < 0) return fail(s, PBD_ERR_INVALID_ARGUMENT, "particle %u has negative phase", i);
        if (phase[i] == PBD_PHASE_FLUID) {
            if (!(p[3] > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "fluid particle %u needs inverse mass > 0", i);
            if (rest_density && !(rest_density[i] > 0.f))
                return fail(s, PBD_ERR_INVALID_ARGUMENT, "fluid particle %u needs rest density > 0", i);
            ++nf;
        }
        if (phase[i] == PBD_PHASE_GAS) {
            // createGas refuses fixed particles (simulation.cpp:418-421)
            if (!(p[3] > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "gas particle %u needs inverse mass > 0", i);
            if (rest_density && !(rest_density[i] > 0.f))
                return fail(s, PBD_ERR_INVALID_ARGUMENT, "gas particle %u needs rest density > 0", i);
            ++ng;
        }
        if (phase[i] >= PBD_PHASE_CLOTH) ++nc;
        if (vel)
            for (int k = 0; k < 4; ++k)
                if (!std::isfinite(vel[4ull * i + k])) return fail(s, PBD_ERR_INVALID_ARGUMENT, "particle %u has a non-finite velocity", i);
    }
    const uint32_t off = s->n;
    CUDA_TRY(s, cudaMemcpy(s->x + off, pos_w, n * sizeof(float4), cudaMemcpyHostToDevice));
    if (vel) {
        CUDA_TRY(s, cudaMemcpy(s->v + off, vel, n * sizeof(float4), cudaMemcpyHostToDevice));
    } else {
        CUDA_TRY(s, cudaMemset(s->v + off, 0, n * sizeof(float4)));
    }
    CUDA_TRY(s, cudaMemcpy(s->phase + off, phase, n * 4ull, cudaMemcpyHostToDevice));
    std::vector<float> ro(n, 1.f);
    if (rest_density) std::copy(rest_density, rest_density + n, ro.begin());
    CUDA_TRY(s, cudaMemcpy(s->rho0 + off, ro.data(), n * 4ull, cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(s->x_old + off, pos_w, n * sizeof(float4), cudaMemcpyHostToDevice));
    if (s->batched()) {
        const std::vector<uint16_t> tag(n, (uint16_t)(s->scenes.size() - 1u));
        CUDA_TRY(s, cudaMemcpy(s->d_scene_of + off, tag.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    if (ng && !s->force) {
        CUDA_TRY(s, dalloc(&s->force, s->cap));
        CUDA_TRY(s, dalloc(&s->gas_open, s->cap));
        CUDA_TRY(s, dalloc(&s->glam, s->cap));
        CUDA_TRY(s, cudaMemset(s->force, 0, s->cap * sizeof(float4)));
        CUDA_TRY(s, cudaMemset(s->gas_open, 0, s->cap));
        CUDA_TRY(s, cudaMemset(s->glam, 0, s->cap * sizeof(float)));
    }
    s->n += n;
    s->n_fluid += nf;
    s->n_contact += nc;
    s->n_gas += ng;
    pbd_scene &cur = s->scenes.back();
    cur.count += n;
    cur.n_fluid += nf;
    cur.n_contact += nc;
    cur.n_gas += ng;
    // the shared stencil radius may change; the first gas sets the has-gas flag
    if ((nf && cur.n_fluid == nf) || (ng && s->n_gas == ng))
        if (int rc = refresh_scenes(s)) return rc;
    if (s->n_fluid && !s->vs) CUDA_TRY(s, dalloc(&s->vs, s->cap));
    if (int rc = alloc_list(s)) return rc;
    if (int rc = alloc_skin(s)) return rc;
    s->grid_valid = false;
    ++s->version;
    if (first_index) *first_index = off;
    if (!s->dist_a.empty() || !s->pin_idx.empty()) return upload_constraints(s);
    return PBD_OK;
}

int pbd_add_distance_constraints(pbd_system *s, uint32_t m, const uint32_t *pairs,
                                 const float *rest, const float *stiffness) {
    SYS_GUARD(s);
    if (m == 0) return PBD_OK;
    if (!pairs || !rest) return fail(s, PBD_ERR_INVALID_ARGUMENT, "pairs and rest are required");
    for (uint32_t c = 0; c < m; ++c) {
        if (pairs[2 * c] >= s->n || pairs[2 * c + 1] >= s->n)
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "constraint %u references a particle >= %u", c, s->n);
        if (pairs[2 * c] == pairs[2 * c + 1])
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "constraint %u joins a particle to itself", c);
        if (s->batched() && scene_of_slot(s, pairs[2 * c]) != scene_of_slot(s, pairs[2 * c + 1]))
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "constraint %u joins particles of different scenes", c);
        if (!std::isfinite(rest[c]) || rest[c] < 0.f)
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "constraint %u has an invalid rest length", c);
        if (stiffness && !(stiffness[c] >= 0.f && stiffness[c] <= 1.f))
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "constraint %u stiffness must be in [0, 1]", c);
    }
    for (uint32_t c = 0; c < m; ++c) {
        s->dist_a.push_back(pairs[2 * c]);
        s->dist_b.push_back(pairs[2 * c + 1]);
        s->dist_rest.push_back(rest[c]);
        s->dist_stiff.push_back(stiffness ? stiffness[c] : 1.f);
    }
    ++s->version;
    return upload_constraints(s);
}

int pbd_add_point_constraints(pbd_system *s, uint32_t p, const uint32_t *index, const float *points) {
    SYS_GUARD(s);
    if (p == 0) return PBD_OK;
    if (!index || !points) return fail(s, PBD_ERR_INVALID_ARGUMENT, "index and points are required");
    for (uint32_t k = 0; k < p; ++k) {
        if (index[k] >= s->n) return fail(s, PBD_ERR_INVALID_ARGUMENT, "pin %u references a particle >= %u", k, s->n);
        for (int d = 0; d < 3; ++d)
            if (!std::isfinite(points[3 * k + d])) return fail(s, PBD_ERR_INVALID_ARGUMENT, "pin %u point is not finite", k);
    }
    for (uint32_t k = 0; k < p; ++k) {
        s->pin_idx.push_back(index[k]);
        for (int d = 0; d < 3; ++d) s->pin_pts.push_back(points[3 * k + d]);
    }
    ++s->version;
    return upload_constraints(s);
}

// Uploads the signed-distance data and the particle -> body map (the map is
// rebuilt from the body ranges; particles without data keep depth -1).
static int upload_sdf(pbd_system *s) {
    if (!s->sdf) {
        CUDA_TRY(s, dalloc(&s->sdf, s->cap));
        CUDA_TRY(s, dalloc(&s->body_of, s->cap));
        const std::vector<float4> none(s->cap, make_float4(0.f, 0.f, 0.f, -1.f));
        CUDA_TRY(s, cudaMemcpy(s->sdf, none.data(), s->cap * sizeof(float4), cudaMemcpyHostToDevice));
    }
    std::vector<int> body(s->cap, -1);
    for (size_t b = 0; b < s->body_range.size(); ++b)
        for (uint32_t k = 0; k < s->body_range[b].y; ++k) body[s->body_range[b].x + k] = (int)b;
    CUDA_TRY(s, cudaMemcpy(s->body_of, body.data(), s->cap * sizeof(int), cudaMemcpyHostToDevice));
    if (!s->sdf_host.empty())
        CUDA_TRY(s, cudaMemcpy(s->sdf, s->sdf_host.data(), s->sdf_host.size() * sizeof(float4), cudaMemcpyHostToDevice));
    return PBD_OK;
}

int pbd_set_rigid_sdf(pbd_system *s, uint32_t body, const float *sdf) {
    SYS_GUARD(s);
    if (body >= s->body_range.size()) return fail(s, PBD_ERR_INVALID_ARGUMENT, "no rigid body %u", body);
    if (!sdf) return fail(s, PBD_ERR_INVALID_ARGUMENT, "sdf is NULL");
    const uint4 r = s->body_range[body];
    std::vector<float4> val(r.y);
    for (uint32_t k = 0; k < r.y; ++k) {
        const float *e = sdf + 4ull * k;
        if (!std::isfinite(e[0]) || !std::isfinite(e[1]) || !std::isfinite(e[2]) || !std::isfinite(e[3]))
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "sdf entry %u is not finite", k);
        if (e[3] < 0.f) {
            val[k] = make_float4(0.f, 0.f, 0.f, -1.f);
            continue;
        }
        const double len = std::sqrt((double)e[0] * e[0] + (double)e[1] * e[1] + (double)e[2] * e[2]);
        if (!(len > 0.0)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "sdf entry %u has a zero normal", k);
        val[k] = make_float4((float)(e[0] / len), (float)(e[1] / len), (float)(e[2] / len), e[3]);
    }
    if (s->sdf_host.size() < s->n) s->sdf_host.resize(s->n, make_float4(0.f, 0.f, 0.f, -1.f));
    std::copy(val.begin(), val.end(), s->sdf_host.begin() + r.x);
    CUDA_TRY(s, cudaDeviceSynchronize());
    if (int rc = upload_sdf(s)) return rc;
    const bool first = !s->any_sdf;
    s->any_sdf = true;
    if (first)
        if (int rc = refresh_scenes(s)) return rc;
    ++s->version;
    return PBD_OK;
}

int pbd_add_rigid_body(pbd_system *s, uint32_t first, uint32_t count, float stiffness,
                       uint32_t *body_index) {
    SYS_GUARD(s);
    if (count < 2) return fail(s, PBD_ERR_INVALID_ARGUMENT, "a rigid body needs at least 2 particles");
    if ((uint64_t)first + count > s->n) return fail(s, PBD_ERR_INVALID_ARGUMENT, "rigid body range exceeds the particle count");
    if (s->batched() && scene_of_slot(s, first) != scene_of_slot(s, first + count - 1u))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "rigid body spans several scenes");
    if (!(stiffness >= 0.f && stiffness <= 1.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "stiffness must be in [0, 1]");
    for (const uint4 &r : s->body_range)
        if (first < r.x + r.y && r.x < first + count)
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "rigid body overlaps body starting at %u", r.x);
    std::vector<float4> pos(count);
    CUDA_TRY(s, cudaDeviceSynchronize());
    CUDA_TRY(s, cudaMemcpy(pos.data(), s->x + first, count * sizeof(float4), cudaMemcpyDeviceToHost));
    double cx = 0, cy = 0, cz = 0, msum = 0;
    for (uint32_t k = 0; k < count; ++k) {
        if (!(pos[k].w > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "rigid particle %u needs inverse mass > 0", first + k);
        const double m = 1.0 / pos[k].w;
        cx += m * pos[k].x;
        cy += m * pos[k].y;
        cz += m * pos[k].z;
        msum += m;
    }
    cx /= msum;
    cy /= msum;
    cz /= msum;
    const uint32_t roff = (uint32_t)s->body_rest.size();
    for (uint32_t k = 0; k < count; ++k)
        s->body_rest.push_back(make_float4((float)(pos[k].x - cx), (float)(pos[k].y - cy),
                                           (float)(pos[k].z - cz), (float)(1.0 / pos[k].w)));
    // keep the rotations of existing bodies
    std::vector<float4> quats(s->body_range.size() + 1, make_float4(0.f, 0.f, 0.f, 1.f));
    if (s->bodies.count)
        CUDA_TRY(s, cudaMemcpy(quats.data(), s->bodies.quat, s->bodies.count * sizeof(float4), cudaMemcpyDeviceToHost));
    s->body_range.push_back(make_uint4(first, count, roff, 0));
    s->body_stiff.push_back(stiffness);
    if (body_index) *body_index = (uint32_t)s->body_range.size() - 1u;
    ++s->version;
    if (int rc = upload_bodies(s, quats)) return rc;
    return s->sdf ? upload_sdf(s) : PBD_OK;
}

static int copy_state(pbd_system *s, float4 *buf, uint32_t first, uint32_t count, float *host_or_dev,
                      int on_device, void *stream, bool to_sys) {
    SYS_GUARD(s);
    if ((uint64_t)first + count > s->n) return fail(s, PBD_ERR_INVALID_ARGUMENT, "range exceeds particle count %u", s->n);
    if (count == 0) return PBD_OK;
    if (!host_or_dev) return fail(s, PBD_ERR_INVALID_ARGUMENT, "buffer is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = (size_t)count * sizeof(float4);
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : (to_sys ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    if (to_sys) CUDA_TRY(s, cudaMemcpyAsync(buf + first, host_or_dev, bytes, kind, st));
    else CUDA_TRY(s, cudaMemcpyAsync(host_or_dev, buf + first, bytes, kind, st));
    if (!on_device) CUDA_TRY(s, cudaStreamSynchronize(st));
    if (to_sys) s->grid_valid = false;
    return PBD_OK;
}

int pbd_set_positions(pbd_system *s, uint32_t first, uint32_t count, const float *src, int on_dev, void *st) {
    return copy_state(s, s ? s->x : nullptr, first, count, const_cast<float *>(src), on_dev, st, true);
}
int pbd_set_velocities(pbd_system *s, uint32_t first, uint32_t count, const float *src, int on_dev, void *st) {
    return copy_state(s, s ? s->v : nullptr, first, count, const_cast<float *>(src), on_dev, st, true);
}
int pbd_get_positions(pbd_system *s, uint32_t first, uint32_t count, float *dst, int on_dev, void *st) {
    return copy_state(s, s ? s->x : nullptr, first, count, dst, on_dev, st, false);
}
int pbd_get_velocities(pbd_system *s, uint32_t first, uint32_t count, float *dst, int on_dev, void *st) {
    return copy_state(s, s ? s->v : nullptr, first, count, dst, on_dev, st, false);
}

// Positions and velocities copied concurrently: x on the caller's stream,
// v on the system's side stream, forked from and joined back into the
// caller's stream with events (so the pair is ordered like one operation
// on that stream); for host memory the call returns after both.
static int copy_pair(pbd_system *s, uint32_t first, uint32_t count, float *x, float *v, int on_device,
                     void *stream, bool to_sys) {
    SYS_GUARD(s);
    if ((uint64_t)first + count > s->n) return fail(s, PBD_ERR_INVALID_ARGUMENT, "range exceeds particle count %u", s->n);
    if (count == 0 || (!x && !v)) return PBD_OK;
    if (!x || !v) {  // one of the two: the plain copy
        return copy_state(s, x ? s->x : s->v, first, count, x ? x : v, on_device, stream, to_sys);
    }
    if (!s->copy_stream) CUDA_TRY(s, cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    if (!s->copy_fork) CUDA_TRY(s, cudaEventCreateWithFlags(&s->copy_fork, cudaEventDisableTiming));
    if (!s->copy_join) CUDA_TRY(s, cudaEventCreateWithFlags(&s->copy_join, cudaEventDisableTiming));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = (size_t)count * sizeof(float4);
    const cudaMemcpyKind kind =
        on_device ? cudaMemcpyDeviceToDevice : (to_sys ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
    CUDA_TRY(s, cudaEventRecord(s->copy_fork, st));
    CUDA_TRY(s, cudaStreamWaitEvent(s->copy_stream, s->copy_fork, 0));
    if (to_sys) {
        CUDA_TRY(s, cudaMemcpyAsync(s->x + first, x, bytes, kind, st));
        CUDA_TRY(s, cudaMemcpyAsync(s->v + first, v, bytes, kind, s->copy_stream));
    } else {
        CUDA_TRY(s, cudaMemcpyAsync(x, s->x + first, bytes, kind, st));
        CUDA_TRY(s, cudaMemcpyAsync(v, s->v + first, bytes, kind, s->copy_stream));
    }
    CUDA_TRY(s, cudaEventRecord(s->copy_join, s->copy_stream));
    CUDA_TRY(s, cudaStreamWaitEvent(st, s->copy_join, 0));
    if (!on_device) CUDA_TRY(s, cudaStreamSynchronize(st));
    if (to_sys) s->grid_valid = false;
    return PBD_OK;
}

int pbd_set_positions_velocities(pbd_system *s, uint32_t first, uint32_t count, const float *x, const float *v,
                                 int on_device, void *stream) {
    return copy_pair(s, first, count, const_cast<float *>(x), const_cast<float *>(v), on_device, stream, true);
}
int pbd_get_positions_velocities(pbd_system *s, uint32_t first, uint32_t count, float *x, float *v, int on_device,
                                 void *stream) {
    return copy_pair(s, first, count, x, v, on_device, stream, false);
}

int pbd_get_vbo(pbd_system *s, uint32_t first, uint32_t count, float *dst, int on_dev, void *stream) {
    SYS_GUARD(s);
    if ((uint64_t)first + count > s->n) return fail(s, PBD_ERR_INVALID_ARGUMENT, "range exceeds particle count %u", s->n);
    if (count == 0) return PBD_OK;
    if (!dst) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dst is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    if (on_dev) {
        CUDA_TRY(s, pbd::launch_vbo(count, s->x + first, (float4 *)dst, st));
        return PBD_OK;
    }
    CUDA_TRY(s, cudaMemcpyAsync(dst, s->x + first, (size_t)count * sizeof(float4), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(s, cudaStreamSynchronize(st));
    for (uint32_t k = 0; k < count; ++k) dst[4 * (size_t)k + 3] = 1.f;
    return PBD_OK;
}

int pbd_get_phases(pbd_system *s, int32_t *dst) {
    SYS_GUARD(s);
    if (!dst) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dst is NULL");
    CUDA_TRY(s, cudaDeviceSynchronize());
    if (s->n) CUDA_TRY(s, cudaMemcpy(dst, s->phase, s->n * 4ull, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_add_fluid_group(pbd_system *s, uint32_t first, uint32_t count, float rest_density) {
    SYS_GUARD(s);
    if ((uint64_t)first + count > s->n)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "range [%u, %u) exceeds the %u particles", first, first + count, s->n);
    if (!(rest_density > 0.f) || !std::isfinite(rest_density))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "rest density must be finite and > 0");
    if (count == 0) return PBD_OK;
    CUDA_TRY(s, cudaDeviceSynchronize());
    std::vector<int32_t> ph(count);
    std::vector<float4> pos(count);
    CUDA_TRY(s, cudaMemcpy(ph.data(), s->phase + first, count * 4ull, cudaMemcpyDeviceToHost));
    CUDA_TRY(s, cudaMemcpy(pos.data(), s->x + first, count * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < count; ++k) {
        if (!(pos[k].w > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "fluid particle %u needs inverse mass > 0", first + k);
        for (const uint4 &r : s->body_range)
            if (first + k >= r.x && first + k < r.x + r.y)
                return fail(s, PBD_ERR_INVALID_ARGUMENT, "particle %u belongs to a rigid body", first + k);
    }
    // the phase census of every scene the range touches
    for (uint32_t k = 0; k < count; ++k) {
        pbd_scene &sc = s->scenes[s->batched() ? scene_of_slot(s, first + k) : 0];
        const int p = ph[k];
        if (p == PBD_PHASE_FLUID) continue;
        if (p == PBD_PHASE_GAS) { --s->n_gas; --sc.n_gas; }
        if (p >= PBD_PHASE_CLOTH) { --s->n_contact; --sc.n_contact; }
        ++s->n_fluid;
        ++sc.n_fluid;
    }
    const std::vector<int32_t> fluid(count, PBD_PHASE_FLUID);
    const std::vector<float> ro(count, rest_density);
    CUDA_TRY(s, cudaMemcpy(s->phase + first, fluid.data(), count * 4ull, cudaMemcpyHostToDevice));
    CUDA_TRY(s, cudaMemcpy(s->rho0 + first, ro.data(), count * 4ull, cudaMemcpyHostToDevice));
    if (int rc = refresh_scenes(s)) return rc;
    if (s->n_fluid && !s->vs) CUDA_TRY(s, dalloc(&s->vs, s->cap));
    if (int rc = alloc_list(s)) return rc;
    if (int rc = alloc_skin(s)) return rc;
    s->grid_valid = false;
    s->list_valid = false;
    ++s->version;
    return PBD_OK;
}

int pbd_add_rigid_group(pbd_system *s, uint32_t first, uint32_t count, float stiffness) {
    return pbd_add_rigid_body(s, first, count, stiffness, nullptr);
}

int pbd_set_box(pbd_system *s, const float box_min[3], const float box_max[3]) {
    SYS_GUARD(s);
    if (!box_min || !box_max) return fail(s, PBD_ERR_INVALID_ARGUMENT, "box_min and box_max are required");
    pbd_params p = s->scenes.back().params;
    for (int k = 0; k < 3; ++k) {
        p.box_min[k] = box_min[k];
        p.box_max[k] = box_max[k];
    }
    return pbd_set_scene_params(s, (uint32_t)s->scenes.size() - 1u, &p);
}

int pbd_set_gas_open(pbd_system *s, uint32_t first, uint32_t count, int open) {
    SYS_GUARD(s);
    if ((uint64_t)first + count > s->n)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "range [%u, %u) exceeds the %u particles", first, first + count, s->n);
    if (count == 0 || !s->n_gas) return PBD_OK;
    std::vector<int32_t> ph(count);
    CUDA_TRY(s, cudaDeviceSynchronize());
    CUDA_TRY(s, cudaMemcpy(ph.data(), s->phase + first, count * 4ull, cudaMemcpyDeviceToHost));
    std::vector<uint8_t> flag(count);
    CUDA_TRY(s, cudaMemcpy(flag.data(), s->gas_open + first, count, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < count; ++k)
        if (ph[k] == PBD_PHASE_GAS) flag[k] = open ? 1u : 0u;
    CUDA_TRY(s, cudaMemcpy(s->gas_open + first, flag.data(), count, cudaMemcpyHostToDevice));
    ++s->version;
    return PBD_OK;
}

int pbd_get_forces(pbd_system *s, float *dst) {
    SYS_GUARD(s);
    if (!dst) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dst is NULL");
    CUDA_TRY(s, cudaDeviceSynchronize());
    if (!s->n) return PBD_OK;
    if (s->force) CUDA_TRY(s, cudaMemcpy(dst, s->force, s->n * sizeof(float4), cudaMemcpyDeviceToHost));
    else std::memset(dst, 0, s->n * sizeof(float4));
    return PBD_OK;
}

int pbd_get_device_buffers(pbd_system *s, pbd_device_buffers *out) {
    if (int rc = check_sys(s)) return rc;
    if (!out) return fail(s, PBD_ERR_INVALID_ARGUMENT, "out is NULL");
    out->positions = s->x;
    out->velocities = s->v;
    out->phases = s->phase;
    out->num_particles = s->n;
    out->capacity = s->cap;
    return PBD_OK;
}

// --------------------------------------------------------------- stepping

// splitmix64 output number k (1-based) of the stream started at seed, as a
// U(0, 1) double (53 bits): the generator of the scene builders.
static double splitmix_uniform(uint64_t seed, uint64_t k) {
    uint64_t z = seed + k * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// Recounts the phase census of every scene from the device phases (after
// a kernel changed phases).
static int recount_phases(pbd_system *s) {
    std::vector<int32_t> ph(s->n);
    if (s->n) CUDA_TRY(s, cudaMemcpy(ph.data(), s->phase, s->n * 4ull, cudaMemcpyDeviceToHost));
    s->n_fluid = s->n_contact = s->n_gas = 0;
    for (pbd_scene &sc : s->scenes) {
        sc.n_fluid = sc.n_contact = sc.n_gas = 0;
        for (uint32_t k = sc.first; k < sc.first + sc.count; ++k) {
            sc.n_fluid += ph[k] == PBD_PHASE_FLUID;
            sc.n_gas += ph[k] == PBD_PHASE_GAS;
            sc.n_contact += ph[k] >= PBD_PHASE_CLOTH;
        }
        s->n_fluid += sc.n_fluid;
        s->n_gas += sc.n_gas;
        s->n_contact += sc.n_contact;
    }
    return refresh_scenes(s);
}

int pbd_add_emitter(pbd_system *s, const pbd_emitter *e, uint32_t *id) {
    SYS_GUARD(s);
    if (!e) return fail(s, PBD_ERR_INVALID_ARGUMENT, "emitter is NULL");
    if (!(e->rate > 0.f) || !std::isfinite(e->rate)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "rate must be > 0");
    if (e->phase != PBD_PHASE_FLUID && e->phase != PBD_PHASE_GAS)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "an emitter emits fluid or gas");
    if (!(e->inverse_mass > 0.f) || !(e->rest_density > 0.f))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "inverse_mass and rest_density must be > 0");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(e->position[k]) || !std::isfinite(e->velocity[k]) || !std::isfinite(e->velocity_jitter[k]))
            return fail(s, PBD_ERR_INVALID_ARGUMENT, "emitter position and velocity must be finite");
    if ((uint64_t)e->group_first + e->group_count > s->n)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "solidification group exceeds the particle count");
    if (e->solidify) {
        if (!s->solid_timer) {
            CUDA_TRY(s, dalloc(&s->solid_timer, s->cap));
            CUDA_TRY(s, dalloc(&s->solid_tag, s->cap));
            CUDA_TRY(s, dalloc(&s->solid_count, 1));
            CUDA_TRY(s, dalloc(&s->solid_list, s->cap));
            const std::vector<float> four(s->cap, 4.f);
            CUDA_TRY(s, cudaMemcpy(s->solid_timer, four.data(), s->cap * 4ull, cudaMemcpyHostToDevice));
            CUDA_TRY(s, cudaMemset(s->solid_tag, 0, s->cap));
        }
        if (e->group_count) CUDA_TRY(s, cudaMemset(s->solid_tag + e->group_first, 1, e->group_count));
    }
    s->emitters.push_back(pbd_system::Emitter{*e});
    if (id) *id = (uint32_t)s->emitters.size() - 1u;
    return PBD_OK;
}

int pbd_emit(pbd_system *s, float dt, uint32_t *emitted, void *stream) {
    SYS_GUARD(s);
    if (emitted) *emitted = 0;
    if (!(dt >= 0.f) || !std::isfinite(dt)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be >= 0");
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(s, cudaStreamSynchronize(st));
    // solidification first (the reference's order), on the last update's
    // grid and lambdas; only where both exist
    bool any_solid = false;
    float speed = 0.f, height = 0.f;
    for (const auto &e : s->emitters)
        if (e.spec.solidify) {
            any_solid = true;
            speed = e.spec.solidify_speed;
            height = e.spec.solidify_height;
        }
    if (any_solid && s->grid_valid && s->n_fluid && s->n) {
        CUDA_TRY(s, cudaMemsetAsync(s->solid_count, 0, 4, st));
        CUDA_TRY(s, pbd::launch_solidify(s->n, dt, speed, height, s->grid.sorted_idx, s->sxl, s->solid_tag,
                                         s->solid_timer, s->x, s->x_old, s->v, s->phase, s->force, s->solid_count,
                                         s->solid_list, st));
        uint32_t converted = 0;
        CUDA_TRY(s, cudaMemcpyAsync(&converted, s->solid_count, 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(s, cudaStreamSynchronize(st));
        if (converted) {
            // pin each new solid where it stopped (in index order, so the
            // constraint order does not depend on the kernel's atomics)
            std::vector<uint32_t> idx(converted);
            CUDA_TRY(s, cudaMemcpy(idx.data(), s->solid_list, converted * 4ull, cudaMemcpyDeviceToHost));
            std::sort(idx.begin(), idx.end());
            std::vector<float> pts(3ull * converted);
            for (uint32_t k = 0; k < converted; ++k) {
                float4 p;
                CUDA_TRY(s, cudaMemcpy(&p, s->x + idx[k], sizeof(float4), cudaMemcpyDeviceToHost));
                pts[3 * k] = p.x;
                pts[3 * k + 1] = p.y;
                pts[3 * k + 2] = p.z;
            }
            if (int rc = recount_phases(s)) return rc;
            if (int rc = pbd_add_point_constraints(s, converted, idx.data(), pts.data())) return rc;
            s->grid_valid = false;
            s->list_valid = false;
            ++s->version;
        }
    }
    uint32_t total = 0;
    for (auto &e : s->emitters) {
        const pbd_emitter &sp = e.spec;
        e.timer += dt;
        e.elapsed += dt;
        uint32_t due = 0;
        const double period = 1.0 / sp.rate;
        while ((sp.duration <= 0.f || e.elapsed < sp.duration) && e.timer >= period) {
            e.timer -= period;
            ++due;
        }
        due = std::min<uint32_t>(due, s->cap - s->n);
        if (!due) continue;
        std::vector<float4> pos(due), vel(due);
        for (uint32_t k = 0; k < due; ++k) {
            pos[k] = make_float4(sp.position[0], sp.position[1], sp.position[2], sp.inverse_mass);
            float u[3];
            for (int a = 0; a < 3; ++a) u[a] = (float)splitmix_uniform(sp.seed, ++e.draws);
            vel[k] = make_float4(sp.velocity[0] + u[0] * sp.velocity_jitter[0],
                                 sp.velocity[1] + u[1] * sp.velocity_jitter[1],
                                 sp.velocity[2] + u[2] * sp.velocity_jitter[2], 0.f);
        }
        const std::vector<int32_t> ph(due, sp.phase);
        const std::vector<float> ro(due, sp.rest_density);
        uint32_t first = 0;
        if (int rc = pbd_add_particles(s, due, &pos[0].x, &vel[0].x, ph.data(), ro.data(), &first)) return rc;
        if (sp.phase == PBD_PHASE_GAS && sp.open_gas)
            if (int rc = pbd_set_gas_open(s, first, due, 1)) return rc;
        if (sp.solidify) CUDA_TRY(s, cudaMemset(s->solid_tag + first, 1, due));
        total += due;
    }
    if (emitted) *emitted = total;
    return PBD_OK;
}

int pbd_tick(pbd_system *s, float dt, void *stream) { return pbd_update(s, dt, stream); }

int pbd_batch_tick(pbd_system *s, float dt, uint32_t nsteps, void *stream) {
    return pbd_update_graph(s, dt, nsteps, stream);
}

int pbd_update(pbd_system *s, float dt, void *stream) {
    SYS_GUARD(s);
    if (!(dt > 0.f) || !std::isfinite(dt)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (s->n == 0) return PBD_OK;
    return enqueue_update(s, clamp_dt(s, dt), (cudaStream_t)stream);
}

int pbd_update_graph(pbd_system *s, float dt, uint32_t nsteps, void *stream) {
    SYS_GUARD(s);
    if (!(dt > 0.f) || !std::isfinite(dt)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (s->n == 0 || nsteps == 0) return PBD_OK;
    dt = clamp_dt(s, dt);
    cudaStream_t st = (cudaStream_t)stream;
    if (!s->graph_exec || s->graph_dt != dt || s->graph_version != s->version) {
        drop_graph(s);
        if (!s->graph_stream) CUDA_TRY(s, cudaStreamCreateWithFlags(&s->graph_stream, cudaStreamNonBlocking));
        // capture on a private stream, ordered after the caller's work
        CUDA_TRY(s, cudaStreamSynchronize(st));
        CUDA_TRY(s, cudaStreamBeginCapture(s->graph_stream, cudaStreamCaptureModeThreadLocal));
        const uint64_t launches0 = s->launches, steps0 = s->steps;
        s->capturing = true;
        int rc = enqueue_update(s, dt, s->graph_stream);
        s->capturing = false;
        s->graph_kernels = s->launches - launches0;
        s->launches = launches0;  // counted when replayed
        s->steps = steps0;
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(s->graph_stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return fail(s, PBD_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&s->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            s->graph_exec = nullptr;
            return fail(s, PBD_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ce));
        }
        s->graph_dt = dt;
        s->graph_version = s->version;
    }
    for (uint32_t k = 0; k < nsteps; ++k) CUDA_TRY(s, cudaGraphLaunch(s->graph_exec, st));
    s->launches += s->graph_kernels * nsteps;
    s->steps += nsteps;
    s->grid_valid = true;
    return PBD_OK;
}

int pbd_set_tuning(pbd_system *s, const pbd_tuning *t) {
    if (int rc = check_sys(s)) return rc;
    if (!t) return fail(s, PBD_ERR_INVALID_ARGUMENT, "tuning is NULL");
    const uint32_t k = t->threads_per_particle;
    if (!(k == 1 || k == 2 || k == 4 || k == 8 || k == 16 || k == 32))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "threads_per_particle must be 1, 2, 4, 8, 16 or 32");
    const uint32_t cap = t->neighbor_list_capacity;
    if (cap % 4u || cap > 1024u)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "neighbor_list_capacity must be a multiple of 4, at most 1024");
    if (!(t->neighbor_skin >= 0.f && t->neighbor_skin <= 1.f))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "neighbor_skin must be in [0, 1]");
    if (t->list_assembly > 1u) return fail(s, PBD_ERR_INVALID_ARGUMENT, "list_assembly must be 0 or 1");
    s->tpp = k;
    s->skin = t->neighbor_skin;
    s->nbl.assemble = t->list_assembly;
    if (int rc = alloc_skin(s)) return rc;
    if (cap != s->list_capacity) {
        free_list(s);
        s->list_capacity = cap;
        if (int rc = alloc_list(s)) return rc;
    }
    s->list_valid = false;
    ++s->version;
    return PBD_OK;
}

int pbd_get_tuning(const pbd_system *s, pbd_tuning *out) {
    if (!s || !out) return PBD_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof *out);
    out->threads_per_particle = s->tpp;
    out->neighbor_list_capacity = s->list_capacity;
    out->neighbor_skin = s->skin;
    out->list_assembly = s->nbl.assemble;
    return PBD_OK;
}

int pbd_autotune(pbd_system *s, float dt, uint32_t steps, void *stream, pbd_tuning *chosen) {
    SYS_GUARD(s);
    if (!(dt > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = s->n;
    if (n == 0 || steps == 0) {
        if (chosen) pbd_get_tuning(s, chosen);
        return PBD_OK;
    }
    dt = clamp_dt(s, dt);
    float4 *snap_x = nullptr, *snap_v = nullptr, *snap_q = nullptr;
    const uint32_t nb = s->bodies.count;
    auto release = [&]() {
        dfree(snap_x);
        dfree(snap_v);
        dfree(snap_q);
    };
    if (dalloc(&snap_x, n) != cudaSuccess || dalloc(&snap_v, n) != cudaSuccess ||
        (nb && dalloc(&snap_q, nb) != cudaSuccess)) {
        release();
        return fail(s, PBD_ERR_CUDA, "autotune: snapshot allocation failed");
    }
    auto copy = [&](bool save) -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(save ? snap_x : s->x, save ? s->x : snap_x, n * sizeof(float4),
                                        cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(save ? snap_v : s->v, save ? s->v : snap_v, n * sizeof(float4),
                                cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess && nb)
            e = cudaMemcpyAsync(save ? snap_q : s->bodies.quat, save ? s->bodies.quat : snap_q,
                                nb * sizeof(float4), cudaMemcpyDeviceToDevice, st);
        return e;
    };
    // candidates: one lane per particle with neighbour lists rebuilt every
    // iteration or kept with a skin of 0.1, 0.2, 0.3 h (list capacity grown
    // with the list volume), the list build without shared memory, the lane groups and,
    // in a system without contacts, cells of half the size (the contact
    // walk's one-cell reach needs the cell of at least the contact
    // distance)
    pbd_tuning base{};
    pbd_get_tuning(s, &base);
    const uint32_t cap0 = base.neighbor_list_capacity ? base.neighbor_list_capacity : 128u;
    std::vector<pbd_tuning> cands;
    std::vector<uint32_t> divs;  // cell divisor of each candidate (0: the given cells on a halved grid)
    auto cand = [&](uint32_t tpp, float skin, uint32_t div = 1u) {
        pbd_tuning t{};
        t.threads_per_particle = tpp;
        t.neighbor_skin = skin;
        const double grow = std::pow(1.0 + (double)skin, 3.0);
        t.neighbor_list_capacity = std::min<uint32_t>(1024u, 4u * (uint32_t)std::ceil(cap0 * grow / 4.0));
        cands.push_back(t);
        divs.push_back(div);
    };
    cand(1, 0.f);
    if (s->n_fluid && base.neighbor_list_capacity)
    {
        cand(1, 0.f);
        cands.back().list_assembly = 1u;
    }
    if (s->n_fluid && s->dev.iterations > 1 && base.neighbor_list_capacity)
        for (float f : {0.1f, 0.2f, 0.3f}) cand(1, f);
    for (uint32_t k : {2u, 4u, 8u, 16u, 32u}) cand(k, 0.f);
    // the scenes' grids as given, and whether halving every cell stays
    // within 2^27 cells
    std::vector<pbd_params> given;
    for (const pbd_scene &sc : s->scenes) given.push_back(sc.params);
    uint64_t half_cells = 0;
    for (const pbd_params &p : given)
        half_cells += (uint64_t)p.grid_size[0] * (p.grid_size[0] > 1u ? 2u : 1u) * p.grid_size[1] *
                      (p.grid_size[1] > 1u ? 2u : 1u) * p.grid_size[2] * (p.grid_size[2] > 1u ? 2u : 1u);
    if (s->any_pbf() && !s->n_contact && half_cells <= (1ull << 27)) cand(1, 0.f, 2u);
    // a grid with many more cells than particles: the same cells on half
    // the grid per axis (the wrap puts more far-away particles in a
    // stencil, which the distance test rejects) where every axis keeps room
    // for its stencil
    uint64_t given_cells = 0;
    bool can_halve = true;
    for (const pbd_params &p : given) {
        given_cells += (uint64_t)p.grid_size[0] * p.grid_size[1] * p.grid_size[2];
        const uint32_t rad = (uint32_t)std::ceil(std::max(p.kernel_radius, 2.f * p.particle_radius) / p.cell_size);
        const bool twod = (p.flags & PBD_FLAG_TWOD) != 0u;
        for (int a = 0; a < 3; ++a)
            if (p.grid_size[a] > 1u && !(twod && a == 2) && p.grid_size[a] / 2u < 2u * rad + 2u) can_halve = false;
    }
    if (can_halve && given_cells > 2ull * n) cand(1, 0.f, 0u);
    uint32_t cur_div = 1u;
    // sets every scene's cells to the given size / div; on a refusal (a
    // parameter limit) puts the given grids back and returns the error
    auto set_div = [&](uint32_t div) -> int {
        if (div == cur_div) return PBD_OK;
        for (uint32_t k = 0; k < (uint32_t)given.size(); ++k) {
            pbd_params p = given[k];
            if (div == 0u) {  // the given cells, half the grid per axis
                const bool twod = (p.flags & PBD_FLAG_TWOD) != 0u;
                for (int a = 0; a < 3; ++a)
                    if (p.grid_size[a] > 1u && !(twod && a == 2)) p.grid_size[a] /= 2u;
            } else {
                p.cell_size = given[k].cell_size / (float)div;
                for (int a = 0; a < 3; ++a)
                    if (p.grid_size[a] > 1u) p.grid_size[a] *= div;
            }
            if (int rc = pbd_set_scene_params(s, k, &p)) {
                for (uint32_t j = 0; j < k; ++j) pbd_set_scene_params(s, j, &given[j]);
                cur_div = 1u;
                return rc;
            }
        }
        cur_div = div;
        return PBD_OK;
    };
    cudaEvent_t a = nullptr, b = nullptr;
    int rc = PBD_OK;
    const bool saved_prof = s->profiling;
    s->profiling = false;
    pbd_tuning best = base;
    uint32_t best_div = 1u;
    float best_ms = 0.f;
    bool have = false;
    if (copy(true) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        rc = fail(s, PBD_ERR_CUDA, "autotune: setup failed");
    }
    for (size_t k = 0; rc == PBD_OK && k < cands.size(); ++k) {
        if (set_div(divs[k]) != PBD_OK) continue;  // a grid the parameters do not allow
        if ((rc = pbd_set_tuning(s, &cands[k])) != PBD_OK) break;
        if (copy(false) != cudaSuccess || (rc = enqueue_update(s, dt, st)) != PBD_OK) break;  // untimed warm-up
        if (copy(false) != cudaSuccess) break;
        cudaEventRecord(a, st);
        for (uint32_t i = 0; i < steps && rc == PBD_OK; ++i) rc = enqueue_update(s, dt, st);
        cudaEventRecord(b, st);
        float ms = 0.f;
        if (rc || cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
            if (!rc) rc = fail(s, PBD_ERR_CUDA, "autotune: timing failed");
            break;
        }
        // a change of grid has to win by 3 % (it changes the user's grid)
        const float bar = divs[k] != 1u ? 0.97f : 1.f;
        if (!have || ms < best_ms * bar) {
            best_ms = ms;
            best = cands[k];
            best_div = divs[k];
            have = true;
        }
    }
    if (copy(false) != cudaSuccess && !rc) rc = fail(s, PBD_ERR_CUDA, "autotune: restore failed");
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = fail(s, PBD_ERR_CUDA, "autotune: sync failed");
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    release();
    s->profiling = saved_prof;
    const int rc3 = set_div(rc ? 1u : best_div);
    const int rc2 = pbd_set_tuning(s, rc ? &base : &best);
    if (!rc) rc = rc3 ? rc3 : rc2;
    s->grid_valid = false;
    ++s->version;
    if (chosen) pbd_get_tuning(s, chosen);
    return rc;
}

int pbd_list_reuses(pbd_system *s, uint32_t *count) {
    SYS_GUARD(s);
    if (!count) return fail(s, PBD_ERR_INVALID_ARGUMENT, "count is NULL");
    *count = 0;
    if (!s->skin_words || !(s->skin > 0.f)) return PBD_OK;
    CUDA_TRY(s, cudaDeviceSynchronize());
    CUDA_TRY(s, cudaMemcpy(count, s->skin_words + pbd::kSkinWords - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_set_profiling(pbd_system *s, int enable) {
    if (int rc = check_sys(s)) return rc;
    s->profiling = enable != 0;
    return PBD_OK;
}

int pbd_get_profile(pbd_system *s, pbd_profile *out) {
    SYS_GUARD(s);
    if (!out) return fail(s, PBD_ERR_INVALID_ARGUMENT, "out is NULL");
    if (int rc = collect_profile(s)) return rc;
    for (int k = 0; k < PBD_STAGE_COUNT; ++k) {
        out->stage_ms[k] = s->stage_ms[k];
        out->stage_launches[k] = s->stage_launches[k];
    }
    out->kernel_launches = s->launches;
    out->steps = s->steps;
    return PBD_OK;
}

int pbd_reset_profile(pbd_system *s) {
    SYS_GUARD(s);
    if (int rc = collect_profile(s)) return rc;
    for (int k = 0; k < PBD_STAGE_COUNT; ++k) {
        s->stage_ms[k] = 0.0;
        s->stage_launches[k] = 0;
    }
    s->launches = 0;
    s->steps = 0;
    return PBD_OK;
}

int pbd_integrate(pbd_system *s, float dt, void *stream) {
    SYS_GUARD(s);
    if (!(dt > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    CUDA_TRY(s, pbd::launch_predict(s->dev, s->n, clamp_dt(s, dt), s->x, s->v, s->x_old, nullptr,
                                    nullptr, nullptr, (cudaStream_t)stream, s->gas_buffers()));
    s->launches += 1;
    s->grid_valid = false;
    return PBD_OK;
}

int pbd_build_grid(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    return build_grid(s, (cudaStream_t)stream, false);
}

int pbd_collide(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    CUDA_TRY(s, pbd::launch_solve(s->dev, s->n, pbd::kDoContact, 0u, s->grid, s->sxl, s->x_old, s->x, s->nbl,
                                  false, s->tpp, (cudaStream_t)stream, pbd::GasBuffers{}, s->sdf_buffers()));
    s->launches += 1;
    return PBD_OK;
}

int pbd_solve_fluids(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(s, pbd::launch_lambda(s->dev, s->n, 0u, s->grid, s->sxl, s->nbl, s->tpp, st, s->gas_buffers()));
    s->list_valid = s->tpp == 1 && s->nbl.slot != nullptr;
    CUDA_TRY(s, pbd::launch_solve(s->dev, s->n, pbd::kDoFluid, 0u, s->grid, s->sxl, s->x_old, s->x, s->nbl,
                                  s->list_valid, s->tpp, st, s->gas_buffers()));
    s->launches += 2;
    return PBD_OK;
}

int pbd_collide_world(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    CUDA_TRY(s, pbd::launch_solve(s->dev, s->n, pbd::kDoWorld, 0u, s->grid, s->sxl, s->x_old, s->x, s->nbl,
                                  false, s->tpp, (cudaStream_t)stream));
    s->launches += 1;
    return PBD_OK;
}

int pbd_solve_distance_constraints(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    CUDA_TRY(s, pbd::launch_distance(s->dev, 0u, s->cons, s->x, true, false, (cudaStream_t)stream));
    return PBD_OK;
}

int pbd_solve_point_constraints(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    CUDA_TRY(s, pbd::launch_distance(s->dev, 0u, s->cons, s->x, false, true, (cudaStream_t)stream));
    return PBD_OK;
}

int pbd_solve_shapes(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    CUDA_TRY(s, pbd::launch_shapes(s->dev, 0u, s->bodies, s->x, (cudaStream_t)stream));
    return PBD_OK;
}

int pbd_calc_velocity(pbd_system *s, float dt, void *stream) {
    SYS_GUARD(s);
    if (!(dt > 0.f)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    CUDA_TRY(s, pbd::launch_velocity(s->dev, s->n, clamp_dt(s, dt), s->x, s->x_old, s->v, (cudaStream_t)stream));
    return PBD_OK;
}

int pbd_apply_xsph(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    if (!s->vs) return PBD_OK;  // no fluid
    CUDA_TRY(s, pbd::launch_xsph(s->dev, s->n, s->grid, s->v, s->vs, s->nbl, s->list_valid, s->tpp,
                                 (cudaStream_t)stream));
    return PBD_OK;
}

// ------------------------------------------------------------- inspection

int pbd_get_grid(pbd_system *s, uint32_t *sorted_hash, uint32_t *sorted_index, uint32_t *cell_start,
                 uint32_t *cell_end) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    CUDA_TRY(s, cudaDeviceSynchronize());
    const uint32_t n = s->n, cells = s->dev.num_cells;
    std::vector<uint32_t> hash(n), idx(n), first((size_t)cells + 1);
    if (n) {
        CUDA_TRY(s, cudaMemcpy(hash.data(), s->grid.hash, n * 4ull, cudaMemcpyDeviceToHost));
        CUDA_TRY(s, cudaMemcpy(idx.data(), s->grid.sorted_idx, n * 4ull, cudaMemcpyDeviceToHost));
    }
    CUDA_TRY(s, cudaMemcpy(first.data(), s->grid.cell_first, ((size_t)cells + 1) * 4u, cudaMemcpyDeviceToHost));
    for (uint32_t p = 0; p < n; ++p) {
        if (sorted_index) sorted_index[p] = idx[p];
        if (sorted_hash) sorted_hash[p] = hash[idx[p]];
    }
    for (uint32_t c = 0; c < cells; ++c) {
        const bool full = first[c + 1] > first[c];
        if (cell_start) cell_start[c] = full ? first[c] : 0xffffffffu;
        if (cell_end) cell_end[c] = full ? first[c + 1] : 0u;
    }
    return PBD_OK;
}

int pbd_get_lambdas(pbd_system *s, float *dst) {
    SYS_GUARD(s);
    if (int rc = need_grid(s)) return rc;
    if (!dst) return fail(s, PBD_ERR_INVALID_ARGUMENT, "dst is NULL");
    CUDA_TRY(s, cudaDeviceSynchronize());
    const uint32_t n = s->n;
    if (!n) return PBD_OK;
    std::vector<uint32_t> idx(n);
    std::vector<float4> sl(n);
    CUDA_TRY(s, cudaMemcpy(idx.data(), s->grid.sorted_idx, n * 4ull, cudaMemcpyDeviceToHost));
    CUDA_TRY(s, cudaMemcpy(sl.data(), s->sxl, n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t p = 0; p < n; ++p) dst[idx[p]] = sl[p].w;
    if (s->n_gas) {  // gas lambdas live in their own sorted array
        std::vector<float> gl(n);
        std::vector<int32_t> ph(n);
        CUDA_TRY(s, cudaMemcpy(gl.data(), s->glam, n * 4ull, cudaMemcpyDeviceToHost));
        CUDA_TRY(s, cudaMemcpy(ph.data(), s->phase, n * 4ull, cudaMemcpyDeviceToHost));
        for (uint32_t p = 0; p < n; ++p)
            if (ph[idx[p]] == PBD_PHASE_GAS) dst[idx[p]] = gl[p];
    }
    return PBD_OK;
}

int pbd_check_finite(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(s, cudaMemsetAsync(s->flag, 0, 4, st));
    CUDA_TRY(s, pbd::launch_finite_check(s->n, s->x, s->v, s->flag, st));
    uint32_t f = 0;
    CUDA_TRY(s, cudaMemcpyAsync(&f, s->flag, 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(s, cudaStreamSynchronize(st));
    if (f) return fail(s, PBD_ERR_NONFINITE, "non-finite position or velocity");
    return PBD_OK;
}

int pbd_synchronize(pbd_system *s, void *stream) {
    SYS_GUARD(s);
    CUDA_TRY(s, cudaStreamSynchronize((cudaStream_t)stream));
    return PBD_OK;
}

// State blob: header {magic, version, n, bodies}, positions, velocities,
// body rotations.
static const uint32_t kStateMagic = 0x50424431u;  // "PBD1"

// State blob: header {magic, version, n, bodies}, x, v, body rotations and,
// in a system with gas (version 2), the force carried into the next step.
uint64_t pbd_state_size(const pbd_system *s) {
    if (!s) return 0;
    return 16ull + (s->n_gas ? 3ull : 2ull) * s->n * sizeof(float4) + (uint64_t)s->bodies.count * sizeof(float4);
}

int pbd_save_state(pbd_system *s, void *dst, uint64_t size) {
    SYS_GUARD(s);
    if (!dst || size < pbd_state_size(s)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "state buffer too small");
    CUDA_TRY(s, cudaDeviceSynchronize());
    uint32_t hdr[4] = {kStateMagic, s->n_gas ? 2u : 1u, s->n, s->bodies.count};
    char *p = (char *)dst;
    std::memcpy(p, hdr, 16);
    p += 16;
    const size_t pb = (size_t)s->n * sizeof(float4);
    if (pb) {
        CUDA_TRY(s, cudaMemcpy(p, s->x, pb, cudaMemcpyDeviceToHost));
        CUDA_TRY(s, cudaMemcpy(p + pb, s->v, pb, cudaMemcpyDeviceToHost));
    }
    p += 2 * pb;
    if (s->bodies.count)
        CUDA_TRY(s, cudaMemcpy(p, s->bodies.quat, s->bodies.count * sizeof(float4), cudaMemcpyDeviceToHost));
    p += (size_t)s->bodies.count * sizeof(float4);
    if (s->n_gas && pb) CUDA_TRY(s, cudaMemcpy(p, s->force, pb, cudaMemcpyDeviceToHost));
    return PBD_OK;
}

int pbd_load_state(pbd_system *s, const void *src, uint64_t size) {
    SYS_GUARD(s);
    if (!src || size < 16) return fail(s, PBD_ERR_INVALID_ARGUMENT, "state buffer too small");
    uint32_t hdr[4];
    std::memcpy(hdr, src, 16);
    if (hdr[0] != kStateMagic || hdr[1] != (s->n_gas ? 2u : 1u))
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "not a state blob of this system");
    if (hdr[2] != s->n || hdr[3] != s->bodies.count)
        return fail(s, PBD_ERR_INVALID_ARGUMENT, "state blob holds %u particles / %u bodies, system has %u / %u",
                    hdr[2], hdr[3], s->n, s->bodies.count);
    if (size < pbd_state_size(s)) return fail(s, PBD_ERR_INVALID_ARGUMENT, "state buffer too small");
    CUDA_TRY(s, cudaDeviceSynchronize());
    const char *p = (const char *)src + 16;
    const size_t pb = (size_t)s->n * sizeof(float4);
    if (pb) {
        CUDA_TRY(s, cudaMemcpy(s->x, p, pb, cudaMemcpyHostToDevice));
        CUDA_TRY(s, cudaMemcpy(s->v, p + pb, pb, cudaMemcpyHostToDevice));
    }
    p += 2 * pb;
    if (s->bodies.count)
        CUDA_TRY(s, cudaMemcpy(s->bodies.quat, p, s->bodies.count * sizeof(float4), cudaMemcpyHostToDevice));
    p += (size_t)s->bodies.count * sizeof(float4);
    if (s->n_gas && pb) CUDA_TRY(s, cudaMemcpy(s->force, p, pb, cudaMemcpyHostToDevice));
    s->grid_valid = false;
    return PBD_OK;
}

}  // extern "C"
