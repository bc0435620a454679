/*
 * pbd.h -- C ABI of the GB300 (sm_103a) unified position-based-dynamics step.
 *
 * One opaque handle (pbd_system) replaces the reference's ParticleSystem
 * object together with the global thrust vectors its .cu files own
 * (gpu/src/cuda/integration.cu:23-34, shared_variables.cu:8-10,
 * solver.cu:32-41).  Any number of handles may coexist; each handle is used
 * by one host thread at a time.  Every call returns a pbd_status (0 = OK) and
 * never exits the process (the reference's checkCudaErrors exits); the text
 * of the last error is available from pbd_last_error().
 *
 * Array arguments are plain host pointers unless a parameter says otherwise.
 * Positions travel as float4 (x, y, z, inverse mass w), the layout of the
 * reference's position VBO plus its W array (particlesystem.cpp:315-319,
 * shared_variables.cu:71-89).  Stream arguments are cudaStream_t passed as
 * void* (NULL = legacy default stream).
 *
 * Reference interfaces replaced (file:line in ebirenbaum/ParticleSolver):
 *   ParticleSystem class ............ gpu/src/particlesystem.h:22-53
 *   extern "C" device wrappers ...... gpu/src/cuda/wrappers.cuh:10-99
 *   SimParams ........................ gpu/src/cuda/kernel.cuh:9-22
 *   phase constants .................. gpu/src/cuda/shared_variables.cuh:4-9
 */
#ifndef PBD_H
#define PBD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBD_ABI_VERSION 3

typedef enum pbd_status {
    PBD_OK = 0,
    PBD_ERR_INVALID_ARGUMENT = 1, /* bad handle, index, size or parameter   */
    PBD_ERR_CAPACITY = 2,         /* would exceed max_particles (the
                                     reference silently ignored the add,
                                     particlesystem.cpp:311-312,335-336)     */
    PBD_ERR_CUDA = 3,             /* a CUDA runtime call failed              */
    PBD_ERR_STATE = 4,            /* call not valid in the current state    */
    PBD_ERR_NONFINITE = 5,        /* NaN/Inf found by pbd_check_finite       */
    PBD_ERR_UNSUPPORTED = 6       /* feature not available for this scene   */
} pbd_status;

/* Particle phases (gpu/src/cuda/shared_variables.cuh:4-9).  Rigid objects,
 * ropes and cloths use PBD_PHASE_RIGID + object id; particles of one such
 * object never collide with each other (integration_kernel.cuh:336). */
#define PBD_PHASE_FLUID 0
#define PBD_PHASE_GAS 1
#define PBD_PHASE_CLOTH 2
#define PBD_PHASE_SOLID 3
#define PBD_PHASE_RIGID 4

/* Behaviour flags.  With flags == 0 the step reproduces the reference GPU
 * formulas; each flag selects the documented alternative. */
#define PBD_FLAG_TWOD (1u << 0)
/* 2-D mode: the TWOD build of integration_kernel.cuh:111-129 (z walls off,
 * z pinned to twod_z). */
#define PBD_FLAG_DENSITY_NEIGHBOR_MASS (1u << 1)
/* PBF density sums m_j W (cpu totalfluidconstraint.cpp:66) instead of the
 * GPU's own-mass W / w_i (integration_kernel.cuh:577,589). */
#define PBD_FLAG_DELTA_OVER_RHO0 (1u << 2)
/* PBF position delta divided by rho0 (Macklin & Mueller 2013, eq. 12)
 * instead of (rho0 + neighbour count) (integration_kernel.cuh:640). */
#define PBD_FLAG_DISTANCE_MASS_WEIGHTED (1u << 3)
/* Distance correction weighted w_i/(w_i+w_j) (cpu distanceconstraint.cpp:
 * 33-37) instead of 1/2 each (solver_kernel.cuh:53-64). */
#define PBD_FLAG_KERNEL_UNITS (1u << 4)
/* relaxation and s_corr are dimensionless, in kernel-radius units: lambda =
 * -C / (sum |grad C|^2 + relaxation / h^2) and the artificial pressure
 * enters lambda_i + lambda_j + h^2 s_corr.  lambda carries units of
 * length^2 while the published s_corr is a pure number, so without this
 * flag the balance of the two terms depends on the scene's length unit
 * (the reference tuned its literal constants for h = 2,
 * integration_kernel.cuh:25-35,592,634). */
#define PBD_FLAG_SKIP_FIXED_NEIGHBORS (1u << 5)
/* A fluid particle's neighbours leave out fixed particles (w = 0): no
 * density, gradient or correction term and not counted (cpu
 * totalfluidconstraint.cpp:59); the GPU reference counted them. */
#define PBD_FLAG_DELTA_OVER_COUNT (1u << 6)
/* PBF position delta divided by rho0 (n + 1), n the neighbours besides the
 * particle itself -- the CPU reference's delta / p0 / (|neighbours incl.
 * self| + counts) (totalfluidconstraint.cpp:108,114; the counts of other
 * constraints are zero for fluid here) -- instead of (rho0 + n).  Not with
 * PBD_FLAG_DELTA_OVER_RHO0.  With PBD_FLAG_DENSITY_NEIGHBOR_MASS,
 * PBD_FLAG_SKIP_FIXED_NEIGHBORS and solid_density_weight = 0 (S_SOLID) the
 * fluid passes are TotalFluidConstraint::project's. */
#define PBD_FLAG_CPU_CONTACTS (1u << 7)
/* Contacts and walls by the CPU reference's projectors instead of collideD
 * and collide_world_functor: pairs closer than a diameter - 1e-4 (never two
 * fixed particles); two solid-like particles by RigidContactConstraint's
 * plain branch (rigidcontactconstraint.cpp:35-95: the overlap and friction
 * against the start of the step shared by the height-scaled inverse masses
 * w e^y), a solid-like particle touching fluid by ContactConstraint
 * (contactconstraint.cpp:13-42, no friction); each wall passed by
 * BoundaryConstraint (boundaryconstraint.cpp:14-93, x then y then z,
 * friction sqrt(mu) r over (x - x_old) / count); every correction averaged
 * over the particle's contacts and walls (the reference's counts). */
#define PBD_FLAGS_ALL 0xffu

/* Simulation parameters (replaces SimParams, kernel.cuh:9-22, plus the
 * compile-time constants of integration_kernel.cuh:20-42 and
 * particlesystem.cpp:52-66, which become runtime values). */
typedef struct pbd_params {
    float particle_radius;   /* r: contact distance 2.001 r, wall offset r  */
    float kernel_radius;     /* h: PBF smoothing radius (reference H = 2)    */
    float cell_size;         /* grid cell edge (reference 2 r)              */
    uint32_t grid_size[3];   /* cells per axis, each a power of two; cell
                                coordinates wrap (integration_kernel.cuh:
                                197-203)                                    */
    float world_origin[3];   /* grid origin                                 */
    float gravity[3];        /* reference (0, -9.8, 0)                      */
    float box_min[3];        /* world box (reference int3 minBounds)        */
    float box_max[3];        /* world box (reference int3 maxBounds)        */
    uint32_t iterations;     /* solver iterations per update                */
    float max_dt;            /* update() clamps dt (reference 0.05)         */
    float relaxation;        /* lambda denominator epsilon (0.01)           */
    float scorr_k;           /* artificial pressure k (0.1)                 */
    float scorr_n;           /* artificial pressure exponent n (4)          */
    float scorr_dq;          /* artificial pressure dq as a fraction of h   */
    float xsph_c;            /* XSPH viscosity c (0 = off; reference has none) */
    float contact_static_friction;  /* S_FRICTION in collideD (0.005)       */
    float contact_kinetic_friction; /* K_FRICTION in collideD (0.0002)      */
    float wall_static_friction;     /* S_FRICTION under sqrt at walls       */
    float wall_kinetic_friction;    /* K_FRICTION under sqrt at walls       */
    uint32_t max_neighbors;  /* per-particle neighbour cap (500)            */
    float twod_z;            /* z of every particle in PBD_FLAG_TWOD mode   */
    uint32_t flags;          /* PBD_FLAG_*                                  */
    float solid_density_weight; /* weight of a neighbour of phase >= CLOTH in
                                a fluid particle's density and in its own
                                constraint gradient: 1 = the GPU reference
                                (every neighbour counts), 0 = the CPU
                                reference's S_SOLID (totalfluidconstraint.h:
                                30, .cpp:66-68,154); fluid-solid coupling
                                in between (>= 0)                           */
    /* Gas phase (PBD_PHASE_GAS; the CPU reference's GasConstraint,
     * cpu/src/constraint/gasconstraint.cpp:34-134, with its constants from
     * gasconstraint.h:11-21 and simulation.h:21).  Gas particles are PBF
     * particles with their own rest density whose neighbours are the
     * particles with w > 0; a gas particle's correction uses only gas
     * neighbours' lambdas and is divided by (neighbours + 1) rest
     * densities; every iteration it adds the reference's vorticity term
     * (and, in an open gas, the density drag) to a force that the next
     * prediction applies. */
    float gas_gravity_scale; /* gravity on gas particles times this (ALPHA
                                -0.2: gas rises)                            */
    float gas_scorr_k;       /* gas artificial pressure k (K_P 0.2)         */
    float gas_scorr_dq;      /* gas artificial pressure dq / h (DQ_P 0.25)  */
    float gas_solid_density_weight; /* weight of a neighbour of phase >=
                                CLOTH in a gas particle's density (S_SOLID
                                0.5)                                        */
    float gas_drag;          /* open gas: force += v (1 - rho / rho0) *
                                (-gas_drag) per iteration (50)              */
} pbd_params;

typedef struct pbd_system pbd_system;

/* Raw device pointers of one system, for callers that render or post-process
 * in place (the reference mapped its GL VBO, particlesystem.cpp:160). */
typedef struct pbd_device_buffers {
    void *positions;   /* float4[capacity], original particle order */
    void *velocities;  /* float4[capacity]                          */
    void *phases;      /* int32[capacity]                           */
    uint32_t num_particles;
    uint32_t capacity;
} pbd_device_buffers;

/* ---------------------------------------------------------------- setup */

int pbd_abi_version(void);
/* Fills the reference defaults: r 0.25, h 2, cell 2r, grid 64^3, box
 * (-50,0,-50)..(50,200,50), 5 iterations (particleapp.cpp:23-38,
 * particlesystem.cpp:52-66, integration_kernel.cuh:20-42). */
void pbd_default_params(pbd_params *out);
/* Replaces ParticleSystem::ParticleSystem (particlesystem.cpp:36-69). */
int pbd_create(const pbd_params *params, uint32_t max_particles, pbd_system **out);
/* Replaces ParticleSystem::~ParticleSystem / _finalize (particlesystem.cpp:72-134). */
int pbd_destroy(pbd_system *sys);
/* Last error text of sys; sys == NULL gives the calling thread's last
 * pbd_create failure. */
const char *pbd_last_error(const pbd_system *sys);
/* Replaces setParameters (integration.cu:96-100).  With several scenes
 * these act on scene 0. */
int pbd_set_params(pbd_system *sys, const pbd_params *params);
int pbd_get_params(const pbd_system *sys, pbd_params *out);
/* Replaces getNumParticles (particlesystem.h:48). */
uint32_t pbd_num_particles(const pbd_system *sys);
uint32_t pbd_capacity(const pbd_system *sys);

/* ---------------------------------------------------------------- scenes
 *
 * A system holds one or more independent scenes (the reference has one
 * ParticleSystem per scene; particlesystem.cpp:36-69).  pbd_create makes
 * scene 0 with its params; pbd_begin_scene opens the next scene with its
 * own params, and every later pbd_add_* call fills the newest scene.  A
 * scene's particles are the slots [first, first + count) in add order;
 * distance constraints and rigid bodies must stay inside one scene.  Scenes
 * never interact: each has its own grid, box, constants, iteration count
 * and dt clamp (max_dt).  pbd_update advances every scene by one step with
 * the same launches (one per stage over all scenes); a scene with K
 * iterations runs in the last K of the batch's iterations and gives the
 * result it would give alone.  The stage entry points act on every scene
 * with iterations > 0. */
#define PBD_MAX_SCENES 65535u
int pbd_begin_scene(pbd_system *sys, const pbd_params *params, uint32_t *scene_index);
uint32_t pbd_num_scenes(const pbd_system *sys);
/* first / count / params may be NULL. */
int pbd_get_scene(const pbd_system *sys, uint32_t scene, uint32_t *first, uint32_t *count, pbd_params *params);
int pbd_set_scene_params(pbd_system *sys, uint32_t scene, const pbd_params *params);
/* A batch in one call: n_scenes scenes, scene k with params[k] and the next
 * counts[k] particles of pos_w (4 floats each), vel (4 floats each, or
 * NULL), phase (or NULL: fluid) and rest_density (or NULL: 1.0), in scene
 * order -- pbd_create, then pbd_begin_scene and pbd_add_particles per
 * scene.  max_particles: capacity (0 = the sum of counts).  Constraints and
 * bodies are added afterwards by particle index (pbd_get_scene gives each
 * scene's first index).  On failure *out is NULL. */
int pbd_batch_create(uint32_t n_scenes, const pbd_params *params, const uint32_t *counts, const float *pos_w,
                     const float *vel, const int32_t *phase, const float *rest_density, uint32_t max_particles,
                     pbd_system **out);

/* --------------------------------------------------------- scene content */

/* Appends n particles (replaces addParticleMultiple, particlesystem.cpp:
 * 333-348, with appendIntegrationParticle integration.cu:50-72 and
 * appendPhaseAndMass shared_variables.cu:71-89).  pos_w: 4n floats (xyz,
 * inverse mass); vel: 4n floats or NULL (zero); phase: n ints;
 * rest_density: n floats or NULL (1.0).  *first_index receives the index of
 * the first new particle.  Returns PBD_ERR_CAPACITY past max_particles. */
int pbd_add_particles(pbd_system *sys, uint32_t n, const float *pos_w, const float *vel,
                      const int32_t *phase, const float *rest_density, uint32_t *first_index);
/* Distance constraints (replaces addDistanceConstraint, solver.cu:125-156).
 * pairs: 2m particle indices; rest: m lengths; stiffness: m values in
 * [0,1] or NULL (1.0; the reference has no stiffness). */
int pbd_add_distance_constraints(pbd_system *sys, uint32_t m, const uint32_t *pairs,
                                 const float *rest, const float *stiffness);
/* Pins (replaces addPointConstraint, solver.cu:108-123).  points: 3p floats. */
int pbd_add_point_constraints(pbd_system *sys, uint32_t p, const uint32_t *index,
                              const float *points);
/* Shape-matched rigid body over particles [first, first+count) (no GPU
 * counterpart in the reference, whose rigid_body_functor is empty,
 * solver_kernel.cuh:289-312; rest offsets as in the CPU createRigidBody,
 * cpu/src/simulation.cpp:371-406).  Every particle needs w > 0. */
int pbd_add_rigid_body(pbd_system *sys, uint32_t first, uint32_t count, float stiffness,
                       uint32_t *body_index);
/* Signed-distance data of a rigid body's particles for the CPU reference's
 * rigid contact (RigidContactConstraint, cpu/src/constraint/
 * rigidcontactconstraint.cpp:13-96; SDFData, particle.h:82-93): sdf holds 4
 * floats per particle of the body, in the body's rest frame (the frame of
 * its rest offsets): the outward surface direction xyz and the particle's
 * depth below the body's surface (>= 0; < 0 = no data for that particle).
 * In a contact of two particles that both have data, the one nearer its
 * surface supplies the contact normal (rotated by its body's current
 * rotation) and depth, a particle closer than one diameter to the surface
 * takes the normal reflected against the pair direction (initBoundary),
 * and the correction and friction use the CPU solver's height-scaled
 * masses; other contacts keep the particle-particle model.  The gradients
 * are normalised here. */
int pbd_set_rigid_sdf(pbd_system *sys, uint32_t body, const float *sdf);
/* The six uniforms the reference drew from cuRAND for the wall jitter every
 * iteration (integration.cu:326); here an explicit input, default zeros. */
int pbd_set_wall_jitter(pbd_system *sys, const float rands[6]);
/* Overwrite state of particles [first, first+count) (replaces setArray,
 * particlesystem.cpp:701-713).  src_on_device != 0: src is a device pointer
 * and the copy is asynchronous on the stream; otherwise src is host memory
 * and the call returns after the copy (the buffer may be reused at once).
 * The getters likewise: a host dst holds the data when they return. */
int pbd_set_positions(pbd_system *sys, uint32_t first, uint32_t count, const float *src,
                      int src_on_device, void *stream);
int pbd_set_velocities(pbd_system *sys, uint32_t first, uint32_t count, const float *src,
                       int src_on_device, void *stream);
int pbd_get_positions(pbd_system *sys, uint32_t first, uint32_t count, float *dst,
                      int dst_on_device, void *stream);
int pbd_get_velocities(pbd_system *sys, uint32_t first, uint32_t count, float *dst,
                       int dst_on_device, void *stream);
/* Positions and velocities of [first, first+count) in one call (no
 * counterpart in the reference, whose state stayed in its GL buffer): the
 * two copies run concurrently, on the stream and on a side stream of the
 * system ordered after it, so a host that keeps the state in its own memory
 * pays for the slower copy rather than the sum.  Same rules as the single
 * calls: synchronous for host memory, asynchronous on the stream for device
 * pointers; either pointer may be NULL. */
int pbd_set_positions_velocities(pbd_system *sys, uint32_t first, uint32_t count, const float *x,
                                 const float *v, int on_device, void *stream);
int pbd_get_positions_velocities(pbd_system *sys, uint32_t first, uint32_t count, float *x, float *v,
                                 int on_device, void *stream);
int pbd_get_phases(pbd_system *sys, int32_t *dst);
/* The reference's render buffer content (its position VBO, float4 per
 * particle: xyz, w = 1; integration_kernel.cuh:461, particlesystem.cpp:
 * 95-96,160) for particles [first, first+count): count float4 to dst, a
 * device pointer (on the stream) or host memory (synchronous).  Positions
 * keep the inverse mass in w; this is the layout a renderer or trajectory
 * tool written for the reference reads. */
int pbd_get_vbo(pbd_system *sys, uint32_t first, uint32_t count, float *dst, int dst_on_device, void *stream);
/* Marks the gas particles of [first, first+count) as an open gas (open != 0)
 * or a closed one: createGas(..., open) of the CPU reference
 * (simulation.cpp:408-429, gasconstraint.cpp:80).  Non-gas particles in the
 * range are left alone; gas starts closed. */
int pbd_set_gas_open(pbd_system *sys, uint32_t first, uint32_t count, int open);
/* The force every particle carries into the next prediction (4n floats,
 * xyz and 0; the reference's Particle::f, particle.h): vorticity and open
 * drag of gas particles, zero elsewhere.  Synchronous. */
int pbd_get_forces(pbd_system *sys, float *dst);
int pbd_get_device_buffers(pbd_system *sys, pbd_device_buffers *out);

/* Scene builders of the reference class, with its lattice spacings and
 * phases; jitter comes from a seeded splitmix64 stream instead of rand(). */
/* addFluid (particlesystem.cpp:357-405): spacing 2.5 r, phase FLUID. */
int pbd_add_fluid(pbd_system *sys, const int32_t ll[3], const int32_t ur[3], float mass,
                  float density, uint64_t seed);
/* addParticleGrid (particlesystem.cpp:408-458): spacing 2.002 r, SOLID. */
int pbd_add_particle_grid(pbd_system *sys, const int32_t ll[3], const int32_t ur[3],
                          float mass, int jitter, uint64_t seed);
/* addHorizCloth (particlesystem.cpp:461-568). */
int pbd_add_horiz_cloth(pbd_system *sys, const int32_t ll[2], const int32_t ur[2],
                        const float spacing[3], const float dist[2], float mass,
                        int hold_edges);
/* addRope (particlesystem.cpp:570-616). */
int pbd_add_rope(pbd_system *sys, const float start[3], const float spacing[3], float dist,
                 int32_t links, float mass, int pin_start);
/* addStaticSphere (particlesystem.cpp:618-687). */
int pbd_add_static_sphere(pbd_system *sys, const int32_t ll[3], const int32_t ur[3],
                          float spacing);

/* The entry points under the names of the hot-path contract: each forwards
 * to (or is a special case of) one above.  pbd_add_fluid_group makes
 * [first, first+count) fluid with rest density rest_density (the
 * reference's per-particle ros, integration.cu:23-34; every particle needs
 * w > 0); pbd_add_rigid_group is pbd_add_rigid_body without the index;
 * pbd_set_box replaces the world box of the scene being filled (the
 * reference's minBounds / maxBounds, particlesystem.cpp:36-69). */
int pbd_add_fluid_group(pbd_system *sys, uint32_t first, uint32_t count, float rest_density);
int pbd_add_rigid_group(pbd_system *sys, uint32_t first, uint32_t count, float stiffness);
int pbd_set_box(pbd_system *sys, const float box_min[3], const float box_max[3]);

/* Emitters (the CPU reference's FluidEmitter, cpu/src/fluidemitter.cpp:
 * 13-76, and OpenSmokeEmitter, opensmokeemitter.cpp:17-43; the reference
 * GPU path has none).  An emitter appends a particle at `position` every
 * 1 / rate seconds of emitter time while its elapsed time is below
 * `duration` (<= 0: no limit), with velocity `velocity` plus U(0, 1) *
 * velocity_jitter per axis from a seeded splitmix64 stream (the reference
 * fluid emitter: velocity (frand(), 1)), phase FLUID or GAS, the given
 * inverse mass and rest density, gas joining an open gas if open_gas.
 * With solidify, the emitted particles and [group_first, group_first +
 * group_count) take part in the fluid emitter's solidification: a fluid
 * particle slower than solidify_speed at a height <= solidify_height counts
 * its timer (initially 4) down by 1 per emitter tick while its lambda of the
 * last update is <= 0, and up by dt (to 3 at most) while it is > 0; at 0 it
 * becomes a fixed solid (phase SOLID, inverse mass 0, at rest), held where
 * it stopped by a point constraint (as the reference GPU holds its static
 * particles, particlesystem.cpp:672-681).  The
 * reference's smoke emitter also advected drawing-only tracer particles;
 * they take no part in the simulation and are not built. */
typedef struct pbd_emitter {
    float position[3];
    float rate;              /* particles per second                        */
    float duration;          /* seconds of emission (FluidEmitter: 5)       */
    int32_t phase;           /* PBD_PHASE_FLUID or PBD_PHASE_GAS            */
    float inverse_mass;      /* of an emitted particle (reference: 1)       */
    float rest_density;
    int32_t open_gas;
    float velocity[3];
    float velocity_jitter[3];
    uint64_t seed;
    int32_t solidify;
    float solidify_speed;    /* reference 0.06                              */
    float solidify_height;   /* reference 5                                 */
    uint32_t group_first, group_count;
} pbd_emitter;

int pbd_add_emitter(pbd_system *sys, const pbd_emitter *emitter, uint32_t *id);
/* Advances every emitter by dt -- the reference ticks its emitters after
 * each simulation step (simulation.cpp:357-365): appends the particles due
 * (as many as the capacity leaves room for; *emitted receives the number,
 * may be NULL) and runs the solidification on the lambdas of the last
 * update.  Synchronous. */
int pbd_emit(pbd_system *sys, float dt, uint32_t *emitted, void *stream);

/* ------------------------------------------------------------------ step */

/* One simulation step (replaces ParticleSystem::update, particlesystem.cpp:
 * 144-246): predict, then per iteration the grid build, contacts, PBF,
 * walls, distance constraints, pins and shape matching, then the velocity
 * update and XSPH.  Asynchronous on stream. */
int pbd_update(pbd_system *sys, float dt, void *stream);
/* nsteps updates captured once into a CUDA graph and replayed (same
 * results as nsteps pbd_update calls). */
int pbd_update_graph(pbd_system *sys, float dt, uint32_t nsteps, void *stream);
/* pbd_update under the contract's name (ParticleSystem::update = tick). */
int pbd_tick(pbd_system *sys, float dt, void *stream);
/* Every scene of a batched system (pbd_begin_scene) advanced nsteps from a
 * captured CUDA graph: pbd_update_graph under the contract's name. */
int pbd_batch_tick(pbd_system *sys, float dt, uint32_t nsteps, void *stream);

/* Stage entry points, one per reference wrapper (wrappers.cuh:10-99). */
/* integrateSystem (integration.cu:122-135): x_old = x; x += (v + g dt) dt. */
int pbd_integrate(pbd_system *sys, float dt, void *stream);
/* calcHash + sortParticles + reorderDataAndFindCellStart
 * (integration.cu:161-275). */
int pbd_build_grid(pbd_system *sys, void *stream);
/* collide (integration.cu:338-386): contacts with friction, non-fluids. */
int pbd_collide(pbd_system *sys, void *stream);
/* solveFluids (integration.cu:453-508): PBF lambda then delta. */
int pbd_solve_fluids(pbd_system *sys, void *stream);
/* collideWorld (integration.cu:319-336): box walls with friction. */
int pbd_collide_world(pbd_system *sys, void *stream);
/* solveDistanceConstraints (solver.cu:196-231). */
int pbd_solve_distance_constraints(pbd_system *sys, void *stream);
/* solvePointConstraints (solver.cu:180-194). */
int pbd_solve_point_constraints(pbd_system *sys, void *stream);
/* Shape matching of every rigid body (no GPU counterpart in the reference). */
int pbd_solve_shapes(pbd_system *sys, void *stream);
/* calcVelocity (integration.cu:416-426): v = (x - x_old) / dt. */
int pbd_calc_velocity(pbd_system *sys, float dt, void *stream);
/* XSPH viscosity on fluid velocities (not in the reference). */
int pbd_apply_xsph(pbd_system *sys, void *stream);

/* ------------------------------------------------------------ inspection */

/* Grid of the last build in the reference layout (after sortParticles and
 * reorderDataAndFindCellStartD, integration_kernel.cuh:229-299): sorted
 * hashes and particle indices (num_particles each), cell start / end
 * (num cells each; start 0xffffffff and end 0 for empty cells).  Host
 * buffers; any may be NULL. */
int pbd_get_grid(pbd_system *sys, uint32_t *sorted_hash, uint32_t *sorted_index,
                 uint32_t *cell_start, uint32_t *cell_end);
/* PBF lambda of every particle from the last solve, in particle order. */
int pbd_get_lambdas(pbd_system *sys, float *dst);
uint32_t pbd_num_cells(const pbd_system *sys);

/* Neighbour-grid build that allocates nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc where they need a
 * grid -- inside stream capture or a real-time loop, or when every device
 * buffer belongs to the caller's own allocator.  Same result as
 * pbd_build_grid + pbd_get_grid on the same positions: particles sorted by
 * (cell hash, index) and the cell start / end of the reference layout.
 * Inputs and outputs are device pointers the caller owns: positions
 * float4[n] (x, y, z, w), sorted_index uint32[n], cell_start and cell_end
 * uint32[grid cells].  Scratch comes from one fixed device array inside the
 * library (~7 MiB per device, held until the process exits), so n is at
 * most PBD_NOALLOC_MAX_PARTICLES and the grid at most
 * PBD_NOALLOC_MAX_CELLS cells; larger requests return
 * PBD_ERR_INVALID_ARGUMENT.  Each call outside stream capture looks up
 * that array's device address afresh (so a cudaDeviceReset in between is
 * harmless); a call on a capturing stream reuses the address of the last
 * call outside capture, so make the first call on a device before any
 * capture.  Every call shares the array: calls that overlap on the GPU
 * race.  Errors are reported through pbd_last_error(NULL). */
#define PBD_NOALLOC_MAX_PARTICLES (1u << 18)
#define PBD_NOALLOC_MAX_CELLS (1u << 20)
int pbd_build_grid_noalloc(const pbd_params *params, const float *positions, uint32_t n,
                           uint32_t *sorted_index, uint32_t *cell_start, uint32_t *cell_end, void *stream);

/* Returns PBD_ERR_NONFINITE if a position or velocity is NaN/Inf. */
int pbd_check_finite(pbd_system *sys, void *stream);
/* Blocks until the system's work on stream is done. */
int pbd_synchronize(pbd_system *sys, void *stream);

/* --------------------------------------------------------------- tuning */

/* Launch shape of the neighbour passes (no counterpart in the reference,
 * which launched one thread per particle, integration.cu:362,471).  Results
 * do not depend on it beyond FP32 summation order. */
typedef struct pbd_tuning {
    uint32_t threads_per_particle; /* lanes sharing one particle's neighbour
                                      walk: 1, 2, 4, 8, 16 or 32            */
    uint32_t neighbor_list_capacity; /* with threads_per_particle == 1: fluid
                                      neighbours recorded per particle and
                                      iteration (multiple of 4, 0 = no list,
                                      default 256), and a quarter as many row
                                      chunks; particles with more fall back
                                      to the stencil walk                   */
    float neighbor_skin;           /* with a list: its radius is (1 + skin) h
                                      and it is reused by the later
                                      iterations of a step while no particle
                                      has moved more than 0.49 skin h since
                                      it was built (checked on the device
                                      each iteration; else the grid and the
                                      list are rebuilt).  Neighbour sets stay
                                      exact (every use filters |r| < h); only
                                      the summation order differs.  0 = off
                                      (grid and list rebuilt every
                                      iteration, the reference's schedule)  */
    uint32_t list_assembly;        /* with a list: where the lambda pass's
                                      walk keeps a particle's row chunks (a
                                      run of up to 32 candidates of one
                                      stencil row and a bit per neighbour):
                                      0 = the first 12 in shared memory (20
                                      with a skin), the rest in a global
                                      buffer (default); 1 = all in the
                                      global buffer                         */
    uint32_t reserved[4];          /* zero                                  */
} pbd_tuning;

int pbd_set_tuning(pbd_system *sys, const pbd_tuning *tuning);
int pbd_get_tuning(const pbd_system *sys, pbd_tuning *out);
/* Iterations of the last step that reused a skin list (0 without one).
 * Synchronous. */
int pbd_list_reuses(pbd_system *sys, uint32_t *count);
/* Times `steps` updates for each candidate schedule, starting each trial
 * from a device snapshot of the state, then restores the state and keeps
 * the fastest (written to *chosen if not NULL).  Candidates: one lane per
 * particle with lists rebuilt every iteration or kept with a skin of 0.1,
 * 0.2 or 0.3 h, the register list build, 2-32 lanes per particle, in a
 * system with fluid or gas and no contacts cells of half the size (every
 * scene's cell_size halved and grid_size doubled), and in a system with
 * more than twice as many cells as particles the same cells on half the
 * grid per axis (positions wrap onto it as on any grid).  A changed grid is
 * kept only if 3 % faster, and is then visible in pbd_get_params /
 * pbd_get_scene.  Synchronous. */
int pbd_autotune(pbd_system *sys, float dt, uint32_t steps, void *stream, pbd_tuning *chosen);

/* --------------------------------------------------------------- timing */

/* Kernel groups of one step, for the per-stage device timing (no
 * counterpart in the reference, whose only readout was an FPS counter,
 * cpu/src/view.cpp:66,189). */
enum {
    PBD_STAGE_PREDICT = 0,  /* prediction + first cell hash                 */
    PBD_STAGE_GRID = 1,     /* hash, cell offsets, sort into cells, reorder */
    PBD_STAGE_LAMBDA = 2,   /* PBF density / lambda (one kernel)            */
    PBD_STAGE_SOLVE = 3,    /* contacts + PBF delta + walls (one kernel)    */
    PBD_STAGE_DISTANCE = 4, /* distance constraints and pins                */
    PBD_STAGE_SHAPES = 5,   /* shape matching                               */
    PBD_STAGE_VELOCITY = 6, /* velocity update (systems without XSPH)       */
    PBD_STAGE_XSPH = 7,     /* XSPH viscosity; when XSPH runs it also does
                               the velocity update, and VELOCITY stays 0  */
    PBD_STAGE_COUNT = 8
};

typedef struct pbd_profile {
    double stage_ms[PBD_STAGE_COUNT];        /* device time per stage group  */
    uint64_t stage_launches[PBD_STAGE_COUNT]; /* kernels timed per stage     */
    uint64_t kernel_launches;  /* every kernel this system enqueued (graph
                                  replays count each captured kernel)        */
    uint64_t steps;            /* updates enqueued                           */
} pbd_profile;

/* enable != 0: pbd_update brackets each stage group with CUDA events on its
 * stream (eager updates only; captured graphs are not timed). */
int pbd_set_profiling(pbd_system *sys, int enable);
/* Synchronises, then returns the accumulated timings and counters. */
int pbd_get_profile(pbd_system *sys, pbd_profile *out);
int pbd_reset_profile(pbd_system *sys);

/* Checkpoint of the whole dynamic state (positions, velocities, rigid body
 * rotations) as one binary blob. */
uint64_t pbd_state_size(const pbd_system *sys);
int pbd_save_state(pbd_system *sys, void *dst, uint64_t size);
int pbd_load_state(pbd_system *sys, const void *src, uint64_t size);

/* ------------------------------------------------------- differentiation
 *
 * Reverse-mode gradients of a rollout (no counterpart in the reference),
 * through every stage of the step: prediction and the velocity update, the
 * PBF density / lambda solve and its delta (s_corr included), contacts with
 * friction, the world walls (with their friction), distance constraints
 * (including the gradient of each constraint's stiffness), pins, shape
 * matching and XSPH.  Neighbour and contact sets, neighbour counts,
 * friction modes, wall clamps and cut-offs are those of the forward pass,
 * held fixed: the gradient of the piecewise-smooth step where it is smooth
 * (the reference's PBF divisor rho0 + n jumps when a neighbour count
 * changes; PBD_FLAG_DELTA_OVER_RHO0 makes the fluid step smooth).  Rigid
 * bodies' rest shapes are constants.  Works on batched systems. */

/* Replaces the stiffness of every distance constraint, in add order
 * (count = number of constraints; values in [0, 1]; host or device array). */
int pbd_set_distance_stiffness(pbd_system *sys, uint32_t count, const float *stiffness, int on_device,
                               void *stream);
uint32_t pbd_num_distance_constraints(const pbd_system *sys);
/* Runs `steps` updates of dt from the current state (as pbd_update) and
 * keeps the state every `checkpoint_every` steps in device memory for
 * pbd_backward.  Memory: 32 bytes per particle per checkpoint. */
int pbd_rollout(pbd_system *sys, float dt, uint32_t steps, uint32_t checkpoint_every, void *stream);
/* pbd_rollout under the contract's name (the forward pass pbd_backward
 * differentiates). */
int pbd_record(pbd_system *sys, float dt, uint32_t steps, uint32_t checkpoint_every, void *stream);
/* Gradients of a loss L(x_T, v_T) of the last rollout's final state.
 * Device arrays: dL_dx, dL_dv float4[n] (w ignored; NULL = zero);
 * outputs dL_dx0, dL_dv0 float4[n] (w = 0) with respect to the rollout's
 * initial positions and velocities, dL_dstiffness float[m] (add order);
 * any output may be NULL.  Recomputes each checkpoint segment with the
 * forward kernels (working memory (1 + 2 iterations) x checkpoint_every x
 * 16 bytes per particle) and leaves the system in the rollout's final
 * state.  Returns PBD_ERR_STATE if the scene changed since the rollout. */
int pbd_backward(pbd_system *sys, const float *dL_dx, const float *dL_dv, float *dL_dx0, float *dL_dv0,
                 float *dL_dstiffness, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PBD_H */
