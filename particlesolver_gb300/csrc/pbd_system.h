// Host-side state of one pbd_system handle.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pbd.h"
#include "pbd_kernels.h"

// One scene of a system: its parameters, particle range and phase census.
// Scenes are filled in order, so scene k's particles are the slots
// [first, first + count), directly after scene k - 1's.
struct pbd_scene {
    pbd_params params{};
    pbd::DevParams dev{};  // parameter block (cell_base set, no table)
    uint32_t first = 0, count = 0;
    uint32_t n_fluid = 0, n_contact = 0, n_gas = 0;
};

struct pbd_system {
    std::vector<pbd_scene> scenes;  // at least one; particles go to the last
    // Launch parameters: scene 0's block for a single scene; for several,
    // the batch's totals (cell count, most iterations, common stencil
    // radius) with the scene table and the slot -> scene map attached.
    pbd::DevParams dev{};
    pbd::DevParams *d_table = nullptr;  // [scenes] device copy of each scene's block
    uint16_t *d_scene_of = nullptr;     // [cap] scene of each slot (several scenes only)
    uint32_t table_cap = 0;             // entries d_table holds
    uint32_t cap = 0;  // max particles
    uint32_t n = 0;    // live particles
    int device = 0;

    // particle state, original order
    float4 *x = nullptr, *v = nullptr, *x_old = nullptr;
    int *phase = nullptr;
    float *rho0 = nullptr;
    float4 *sxl = nullptr;  // sorted order: position xyz, PBF lambda w
    float4 *vs = nullptr;   // XSPH scratch: velocities in sorted order
    uint32_t *flag = nullptr;  // finite check
    // gas phase (allocated with the first gas particle)
    float4 *force = nullptr;     // force the next prediction applies, original order
    uint8_t *gas_open = nullptr; // 1 = open gas, original order
    float *glam = nullptr;       // gas lambda, sorted order
    // rigid-body signed-distance data (allocated with the first pbd_set_rigid_sdf)
    float4 *sdf = nullptr;       // [cap] rest-frame normal xyz, depth (< 0: none)
    int *body_of = nullptr;      // [cap] body of each particle, -1 for none
    std::vector<float4> sdf_host;  // host copy of sdf for the live particles
    bool any_sdf = false;
    // emitters: host state; solidification timer and membership per particle
    struct Emitter {
        pbd_emitter spec;
        double timer = 0.0, elapsed = 0.0;
        uint64_t draws = 0;  // splitmix64 outputs used so far
    };
    std::vector<Emitter> emitters;
    float *solid_timer = nullptr;   // [cap], starts at 4 (Particle::t)
    uint8_t *solid_tag = nullptr;   // [cap], 1 = takes part in solidification
    uint32_t *solid_count = nullptr;
    uint32_t *solid_list = nullptr; // [cap] particles converted by the last tick

    pbd::GridBuffers grid{};
    uint32_t grid_cells = 0;  // cells the grid arrays were sized for
    bool grid_valid = false;

    // constraints (host lists in add order + device CSR)
    std::vector<uint32_t> dist_a, dist_b;
    std::vector<float> dist_rest, dist_stiff;
    std::vector<uint32_t> pin_idx;
    std::vector<float> pin_pts;
    pbd::ConstraintBuffers cons{};

    // rigid bodies
    std::vector<uint4> body_range;
    std::vector<float> body_stiff;
    std::vector<float4> body_rest;
    pbd::BodyBuffers bodies{};

    // phase census for stage selection (all scenes)
    uint32_t n_fluid = 0, n_contact = 0, n_gas = 0;
    bool any_xsph = false;  // some scene with fluid, xsph_c != 0 and iterations > 0

    uint32_t tpp = 1;     // lanes per particle in the neighbour passes
    pbd::NbList nbl{};    // per-iteration fluid neighbour lists
    uint32_t list_capacity = 256;
    float skin = 0.f;               // skin-list radius (1 + skin) h; 0 = off
    float4 *sref = nullptr;         // [cap] sorted positions at the list build
    uint32_t *skin_words = nullptr; // [pbd::kSkinWords] device decision words
    bool list_valid = false;  // nbl matches the current grid
    int rigid_index = 0;  // next object id for the scene builders
    float rands[6] = {0, 0, 0, 0, 0, 0};

    // stage timing and launch counters
    bool profiling = false;
    bool capturing = false;
    struct TimedStage {
        int stage;
        cudaEvent_t start, stop;
    };
    std::vector<TimedStage> pending;
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[PBD_STAGE_COUNT] = {};
    uint64_t stage_launches[PBD_STAGE_COUNT] = {};
    uint64_t launches = 0;
    uint64_t steps = 0;
    uint64_t graph_kernels = 0;  // kernels in the captured step

    // captured step graph
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t graph_stream = nullptr;
    // side stream and fork / join events of the paired state copies
    // (pbd_set/get_positions_velocities), created on first use
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_fork = nullptr, copy_join = nullptr;
    float graph_dt = 0.f;
    uint64_t graph_version = 0;
    uint64_t version = 1;  // bumped whenever a captured graph would go stale

    // differentiation: checkpoints of the last pbd_rollout and the
    // backward pass's work arrays (pbd_adjoint.cu)
    struct Adjoint {
        bool recorded = false;
        uint64_t version = 0;   // system version the rollout ran on
        float dt = 0.f;
        uint32_t steps = 0, every = 0, nckpt = 0;
        float4 *ckpt_x = nullptr, *ckpt_v = nullptr;  // [nckpt][cap]
        float4 *ckpt_q = nullptr;  // body rotations: [nckpt + 1][bodies] (the last: after the rollout)
        size_t ckpt_q_cap = 0;
        size_t ckpt_cap = 0;                          // states allocated
        float4 *rec = nullptr;                        // segment recording
        size_t rec_cap = 0;                           // states allocated
        float4 *gx = nullptr, *gv = nullptr, *gxo = nullptr, *gt = nullptr, *gy = nullptr, *gu = nullptr;
        float4 *save_x = nullptr, *save_v = nullptr, *save_xo = nullptr;
        float4 *fl1 = nullptr, *fl2 = nullptr, *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;
        float *lbar = nullptr;
        uint32_t *cnt = nullptr;
        float *gstiff = nullptr;
        uint32_t work_cap = 0, stiff_cap = 0;
    } adj;

    std::string err;

    bool batched() const { return scenes.size() > 1; }
    bool any_pbf() const { return n_fluid || n_gas; }
    pbd::GasBuffers gas_buffers() const {
        if (!n_gas) return pbd::GasBuffers{};
        return pbd::GasBuffers{phase, force, gas_open, glam, v, grid.sorted_idx};
    }
    pbd::RigidSdf sdf_buffers() const {
        if (!any_sdf) return pbd::RigidSdf{};
        return pbd::RigidSdf{sdf, body_of, bodies.quat};
    }
    const pbd_params &cur_params() const { return scenes.back().params; }
};

// Shared by the C ABI translation units: parameter validation into device
// constants, and the calling thread's error text for calls without a handle.
int pbd_internal_device_params(const pbd_params *params, pbd::DevParams *out, std::string *why);
void pbd_internal_set_thread_error(const std::string &msg);
// Step internals used by the adjoint (pbd_adjoint.cu).
int pbd_internal_fail(pbd_system *s, int code, const std::string &msg);
int pbd_internal_guard(pbd_system *s);  // handle check + its device current
int pbd_internal_build_grid(pbd_system *s, cudaStream_t st, bool hashed_in_predict);
// rec: the adjoint's recording of the step's positions, or nullptr.
int pbd_internal_enqueue_update(pbd_system *s, float dt, cudaStream_t st, float4 *rec = nullptr);
bool pbd_internal_any_xsph(const pbd_system *s);
float pbd_internal_clamp_dt(const pbd_system *s, float dt);
void pbd_internal_free_adjoint(pbd_system *s);
