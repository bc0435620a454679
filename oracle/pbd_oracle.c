/*
 * pbd_oracle.c -- FP64 CPU restatement of the reference PBD step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (tests/,
 * __graft_entry__.smoke(), bench.py's CPU-baseline leg).  Nothing in the
 * product links or calls it.
 *
 * Follows gpu/src/particlesystem.cpp:144-246 (step order),
 * gpu/src/cuda/integration_kernel.cuh (kernels) and
 * gpu/src/cuda/solver_kernel.cuh + solver.cu (distance constraints, pins);
 * shape matching (absent on the reference GPU) follows the published
 * methods named at orc_solve_shapes.  Deliberate differences from the
 * reference GPU code (the same ones the CUDA path makes) are listed where
 * they occur.  Grid hashes and every neighbour distance test run in FP32
 * with the kernels' rounding sequence; everything else is FP64.
 */
#include "pbd_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* The arithmetic type: double, or (compiled as C++ with ORC_DUAL, see
 * oracle/dual.hpp) a dual number carrying one directional derivative. */
#ifdef ORC_DUAL
#include "dual.hpp"
#else
typedef double real;
#define R_VAL(x) (x)
#endif

#define K_EPS 0.001            /* EPS, integration_kernel.cuh:20        */
#define K_MIN_SPIKY2 1e-8f     /* |r| < 1e-4, integration_kernel.cuh:580,625, decided on |r|^2 */
#define K_MIN_DIST 0.0001      /* solver_kernel.cuh:57                  */
#define K_SHAPE_ITERS 24

struct orc_system {
    pbd_params p;
    uint32_t cap, n, cells;
    int fluid_rad;
    float h2f, collide2f, collidef;
    float cpu_c2f; /* (diameter - EPSILON)^2 in FP32: the CPU contact test */
    double poly6, spiky, poly6_self, scorr_inv_ref, scorr_k, relax, ws, wk;
    double rands[6];
    /* particle state, original order */
    real *x, *v, *x_old;
    double *rho0;
    int32_t *phase;
    /* grid */
    uint32_t *hash, *sorted_idx, *cell_first;
    int grid_valid;
    real *sx;                 /* sorted FP64 positions (4n)               */
    double *srho0;            /* sorted rest densities                    */
    float *sx32;              /* sorted FP32 positions (4n) for the tests  */
    int32_t *sphase;
    real *lambda;             /* sorted order */
    uint32_t *nb_fluid, *nb_contact;  /* original order */
    /* distance constraints (add order) and pins */
    uint32_t m, m_cap, *da, *db;
    double *drest;
    real *dstiff;
    uint32_t npin, pin_cap, *pin_idx;
    double *pin_pts;
    /* rigid bodies */
    uint32_t nb, nb_cap, *bfirst, *bcount;
    double *bstiff;
    real *bquat;              /* 4 per body: x y z w */
    double *brest;            /* 4 per particle of the body: q xyz, mass; indexed by particle */
    /* gas phase (gasconstraint.cpp) */
    int has_gas;
    double gas_scorr_k, gas_scorr_inv_ref;
    real *force;              /* 4n, original order: Particle::f            */
    unsigned char *gas_open;  /* original order                             */
    real *glambda;            /* sorted order                               */
    /* rigid-body signed-distance data (rigidcontactconstraint.cpp) */
    double *sdf;              /* 4 per particle: rest-frame normal, depth (< 0: none) */
    int32_t *body_of;         /* body of each particle, -1 for none          */
    int any_sdf;
};

static int g_threads = 0;

void orc_set_threads(int t) { g_threads = t; }

static void set_threads(void) {
#ifdef _OPENMP
    if (g_threads > 0) omp_set_num_threads(g_threads);
#endif
}

/* ------------------------------------------------------------- helpers */

/* Bit-exact restatement of the kernels' dist2_exact:
 * d2 = fma(dz, dz, fma(dy, dy, dx * dx)) in FP32. */
static inline float dist2f(const float *a, const float *b) {
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    float d = dx * dx;
    d = fmaf(dy, dy, d);
    return fmaf(dz, dz, d);
}

static inline int floor_to_int(float v) {
    float f = floorf(v);
    if (isnan(f)) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

/* calcGridPos + calcGridHash (integration_kernel.cuh:187-203), FP32, IEEE
 * division (the reference built with -use_fast_math; the grid of this
 * project is defined with IEEE division on both sides). */
static inline void grid_cell(const orc_system *s, const float *p, int g[3]) {
    g[0] = floor_to_int((p[0] - s->p.world_origin[0]) / s->p.cell_size);
    g[1] = floor_to_int((p[1] - s->p.world_origin[1]) / s->p.cell_size);
    /* 2-D mode (the TWOD build, integration_kernel.cuh:111-129, pins every
     * particle to twod_z): all particles share twod_z's layer */
    const float z = (s->p.flags & PBD_FLAG_TWOD) ? s->p.twod_z : p[2];
    g[2] = floor_to_int((z - s->p.world_origin[2]) / s->p.cell_size);
}

static inline uint32_t grid_hash(const orc_system *s, const int g[3]) {
    uint32_t x = (uint32_t)g[0] & (s->p.grid_size[0] - 1u);
    uint32_t y = (uint32_t)g[1] & (s->p.grid_size[1] - 1u);
    uint32_t z = (uint32_t)g[2] & (s->p.grid_size[2] - 1u);
    return (z * s->p.grid_size[1] + y) * s->p.grid_size[0] + x;
}

/* Visits the stencil cells around g in the reference's order (z, y, x;
 * integration_kernel.cuh:388-398,549-559), each cell's particles in
 * ascending sorted index.  Calls f(ctx, j); a non-zero return stops. */
typedef int (*visit_fn)(void *ctx, uint32_t j);

static void for_each_candidate(const orc_system *s, const int g[3], int rad, visit_fn f, void *ctx) {
    const uint32_t gx = s->p.grid_size[0], gy = s->p.grid_size[1], gz = s->p.grid_size[2];
    /* in 2-D mode the particles' layer is the only one holding particles */
    const int zr = (s->p.flags & PBD_FLAG_TWOD) ? 0 : rad;
    for (int dz = -zr; dz <= zr; ++dz)
        for (int dy = -rad; dy <= rad; ++dy)
            for (int dx = -rad; dx <= rad; ++dx) {
                uint32_t x = (uint32_t)(g[0] + dx) & (gx - 1u);
                uint32_t y = (uint32_t)(g[1] + dy) & (gy - 1u);
                uint32_t z = (uint32_t)(g[2] + dz) & (gz - 1u);
                uint32_t c = (z * gy + y) * gx + x;
                for (uint32_t j = s->cell_first[c]; j < s->cell_first[c + 1]; ++j)
                    if (f(ctx, j)) return;
            }
}

static void *xrealloc(void *p, size_t bytes) {
    void *q = realloc(p, bytes ? bytes : 1);
    return q;
}

/* ----------------------------------------------------------- lifetime */

orc_system *orc_create(const pbd_params *params, uint32_t cap) {
    orc_system *s = (orc_system *)calloc(1, sizeof *s);
    const double PI = 3.14159265358979323846;
    s->p = *params;
    s->cap = cap;
    s->cells = params->grid_size[0] * params->grid_size[1] * params->grid_size[2];
    const float hf = params->kernel_radius;
    s->h2f = hf * hf;
    s->collidef = params->particle_radius * 2.001f;
    s->collide2f = s->collidef * s->collidef;
    {
        const float c = 2.0f * params->particle_radius - 0.0001f;
        s->cpu_c2f = c * c;
    }
    s->fluid_rad = (int)ceilf(hf / params->cell_size);
    const double h = hf;
    s->poly6 = 315.0 / (64.0 * PI * pow(h, 9.0));
    s->spiky = 45.0 / (PI * pow(h, 6.0));
    s->poly6_self = s->poly6 * pow(h, 6.0);
    const double dq = (double)params->scorr_dq * h, t2 = h * h - dq * dq;
    s->scorr_inv_ref = 1.0 / (s->poly6 * t2 * t2 * t2);
    /* PBD_FLAG_KERNEL_UNITS: s_corr scaled by h^2, relaxation by 1/h^2 */
    const int ku = (params->flags & PBD_FLAG_KERNEL_UNITS) != 0;
    s->scorr_k = ku ? (double)params->scorr_k * h * h : (double)params->scorr_k;
    s->relax = ku ? (double)params->relaxation / (h * h) : (double)params->relaxation;
    s->gas_scorr_k = ku ? (double)params->gas_scorr_k * h * h : (double)params->gas_scorr_k;
    {
        const double gdq = (double)params->gas_scorr_dq * h, gt2 = h * h - gdq * gdq;
        s->gas_scorr_inv_ref = 1.0 / (s->poly6 * gt2 * gt2 * gt2);
    }
    s->ws = sqrt((double)params->wall_static_friction);
    s->wk = sqrt((double)params->wall_kinetic_friction);
    s->x = (real *)calloc(4ull * cap, sizeof(real));
    s->v = (real *)calloc(4ull * cap, sizeof(real));
    s->x_old = (real *)calloc(4ull * cap, sizeof(real));
    s->rho0 = (double *)calloc(cap, sizeof(double));
    s->phase = (int32_t *)calloc(cap, sizeof(int32_t));
    s->hash = (uint32_t *)calloc(cap, sizeof(uint32_t));
    s->sorted_idx = (uint32_t *)calloc(cap, sizeof(uint32_t));
    s->cell_first = (uint32_t *)calloc((size_t)s->cells + 1, sizeof(uint32_t));
    s->sx = (real *)calloc(4ull * cap, sizeof(real));
    s->srho0 = (double *)calloc(cap, sizeof(double));
    s->sx32 = (float *)calloc(4ull * cap, sizeof(float));
    s->sphase = (int32_t *)calloc(cap, sizeof(int32_t));
    s->lambda = (real *)calloc(cap, sizeof(real));
    s->nb_fluid = (uint32_t *)calloc(cap, sizeof(uint32_t));
    s->nb_contact = (uint32_t *)calloc(cap, sizeof(uint32_t));
    s->brest = (double *)calloc(4ull * cap, sizeof(double));
    s->force = (real *)calloc(4ull * cap, sizeof(real));
    s->gas_open = (unsigned char *)calloc(cap ? cap : 1, 1);
    s->glambda = (real *)calloc(cap, sizeof(real));
    s->sdf = (double *)calloc(4ull * (cap ? cap : 1), sizeof(double));
    s->body_of = (int32_t *)malloc((cap ? cap : 1) * sizeof(int32_t));
    for (uint32_t k = 0; k < cap; ++k) {
        s->sdf[4 * k + 3] = -1.0;
        s->body_of[k] = -1;
    }
    return s;
}

void orc_destroy(orc_system *s) {
    if (!s) return;
    free(s->x); free(s->v); free(s->x_old); free(s->rho0); free(s->phase);
    free(s->hash); free(s->sorted_idx); free(s->cell_first);
    free(s->sx); free(s->srho0); free(s->sx32); free(s->sphase); free(s->lambda);
    free(s->nb_fluid); free(s->nb_contact);
    free(s->da); free(s->db); free(s->drest); free(s->dstiff);
    free(s->pin_idx); free(s->pin_pts);
    free(s->bfirst); free(s->bcount); free(s->bstiff); free(s->bquat); free(s->brest);
    free(s->force); free(s->gas_open); free(s->glambda); free(s->sdf); free(s->body_of);
    free(s);
}

int orc_add_particles(orc_system *s, uint32_t n, const double *pos_w, const double *vel,
                      const int32_t *phase, const double *rest_density) {
    if ((uint64_t)s->n + n > s->cap) return PBD_ERR_CAPACITY;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t k = s->n + i;
        for (int d = 0; d < 4; ++d) {
            s->x[4 * k + d] = pos_w[4 * i + d];
            s->x_old[4 * k + d] = pos_w[4 * i + d];
            s->v[4 * k + d] = vel ? vel[4 * i + d] : 0.0;
        }
        s->phase[k] = phase[i];
        s->rho0[k] = rest_density ? rest_density[i] : 1.0;
        if (phase[i] == PBD_PHASE_GAS) s->has_gas = 1;
    }
    s->n += n;
    s->grid_valid = 0;
    return PBD_OK;
}

int orc_add_distance_constraints(orc_system *s, uint32_t m, const uint32_t *pairs, const double *rest,
                                 const double *stiffness) {
    if (s->m + m > s->m_cap) {
        s->m_cap = (s->m + m) * 2;
        s->da = (uint32_t *)xrealloc(s->da, s->m_cap * sizeof(uint32_t));
        s->db = (uint32_t *)xrealloc(s->db, s->m_cap * sizeof(uint32_t));
        s->drest = (double *)xrealloc(s->drest, s->m_cap * sizeof(double));
        s->dstiff = (real *)xrealloc(s->dstiff, s->m_cap * sizeof(real));
    }
    for (uint32_t c = 0; c < m; ++c) {
        s->da[s->m] = pairs[2 * c];
        s->db[s->m] = pairs[2 * c + 1];
        s->drest[s->m] = rest[c];
        s->dstiff[s->m] = stiffness ? stiffness[c] : 1.0;
        ++s->m;
    }
    return PBD_OK;
}

int orc_add_point_constraints(orc_system *s, uint32_t p, const uint32_t *index, const double *points) {
    if (s->npin + p > s->pin_cap) {
        s->pin_cap = (s->npin + p) * 2;
        s->pin_idx = (uint32_t *)xrealloc(s->pin_idx, s->pin_cap * sizeof(uint32_t));
        s->pin_pts = (double *)xrealloc(s->pin_pts, 3ull * s->pin_cap * sizeof(double));
    }
    for (uint32_t k = 0; k < p; ++k) {
        s->pin_idx[s->npin] = index[k];
        for (int d = 0; d < 3; ++d) s->pin_pts[3 * s->npin + d] = points[3 * k + d];
        ++s->npin;
    }
    return PBD_OK;
}

/* Rest offsets q = x - c about the mass-weighted centre, as
 * createRigidBody / Body::updateCOM(useEstimates=false) / computeRs
 * (cpu/src/simulation.cpp:371-406, cpu/src/solver/particle.cpp:15-73). */
int orc_add_rigid_body(orc_system *s, uint32_t first, uint32_t count, double stiffness) {
    if (s->nb + 1 > s->nb_cap) {
        s->nb_cap = (s->nb + 1) * 2;
        s->bfirst = (uint32_t *)xrealloc(s->bfirst, s->nb_cap * sizeof(uint32_t));
        s->bcount = (uint32_t *)xrealloc(s->bcount, s->nb_cap * sizeof(uint32_t));
        s->bstiff = (double *)xrealloc(s->bstiff, s->nb_cap * sizeof(double));
        s->bquat = (real *)xrealloc(s->bquat, 4ull * s->nb_cap * sizeof(real));
    }
    double c[3] = {0, 0, 0}, msum = 0;
    for (uint32_t k = first; k < first + count; ++k) {
        double m = 1.0 / (double)(float)R_VAL(s->x[4 * k + 3]);
        for (int d = 0; d < 3; ++d) c[d] += m * R_VAL(s->x[4 * k + d]);
        msum += m;
    }
    for (int d = 0; d < 3; ++d) c[d] /= msum;
    for (uint32_t k = first; k < first + count; ++k) {
        /* rounded to FP32 like the CUDA path's stored rest offsets */
        for (int d = 0; d < 3; ++d) s->brest[4 * k + d] = (double)(float)(R_VAL(s->x[4 * k + d]) - c[d]);
        s->brest[4 * k + 3] = (double)(float)(1.0 / R_VAL(s->x[4 * k + 3]));
    }
    for (uint32_t k = first; k < first + count; ++k) s->body_of[k] = (int32_t)s->nb;
    s->bfirst[s->nb] = first;
    s->bcount[s->nb] = count;
    s->bstiff[s->nb] = stiffness;
    s->bquat[4 * s->nb + 0] = 0;
    s->bquat[4 * s->nb + 1] = 0;
    s->bquat[4 * s->nb + 2] = 0;
    s->bquat[4 * s->nb + 3] = 1;
    ++s->nb;
    return PBD_OK;
}

void orc_set_wall_jitter(orc_system *s, const double r[6]) {
    for (int k = 0; k < 6; ++k) s->rands[k] = r[k];
}

/* ------------------------------------------------------------- stages */

/* integrate_functor + copyToXstar (integration_kernel.cuh:159-184,
 * shared_variables.cu:91-96).  With gas particles in the system, the CPU
 * reference's step velocity (simulation.cpp:142-153): v' = v + dt g' + dt f
 * with g' = g * gas_gravity_scale on gas (ALPHA, simulation.h:21), f the
 * force of the last step, which is cleared; v' is kept for the gas terms. */
void orc_integrate(orc_system *s, double dt) {
    dt = fmin(dt, (double)s->p.max_dt);
    for (uint32_t i = 0; i < s->n; ++i) {
        for (int d = 0; d < 4; ++d) s->x_old[4 * i + d] = s->x[4 * i + d];
        const double gs = (s->has_gas && s->phase[i] == PBD_PHASE_GAS) ? (double)s->p.gas_gravity_scale : 1.0;
        for (int d = 0; d < 3; ++d) {
            real vv = s->v[4 * i + d] + ((double)s->p.gravity[d] * gs) * dt;
            if (s->has_gas) {
                vv = vv + s->force[4 * i + d] * dt;
                s->v[4 * i + d] = vv;
            }
            s->x[4 * i + d] += vv * dt;
        }
        if (s->has_gas)
            for (int d = 0; d < 4; ++d) s->force[4 * i + d] = 0.0;
    }
    s->grid_valid = 0;
}

/* calcHashD + stable sort by (hash, index) + reorderDataAndFindCellStartD
 * (integration_kernel.cuh:206-299, integration.cu:161-275), as a counting
 * sort: cell_first[c] is the first sorted slot of cell c, so cellStart /
 * cellEnd of a non-empty cell are cell_first[c] / cell_first[c + 1]. */
void orc_build_grid(orc_system *s) {
    const uint32_t n = s->n;
    memset(s->cell_first, 0, ((size_t)s->cells + 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        float p[3] = {(float)R_VAL(s->x[4 * i]), (float)R_VAL(s->x[4 * i + 1]), (float)R_VAL(s->x[4 * i + 2])};
        int g[3];
        grid_cell(s, p, g);
        s->hash[i] = grid_hash(s, g);
        ++s->cell_first[s->hash[i]];
    }
    uint32_t run = 0;
    for (uint32_t c = 0; c <= s->cells; ++c) {
        uint32_t k = s->cell_first[c];
        s->cell_first[c] = run;
        run += k;
    }
    uint32_t *fill = (uint32_t *)calloc((size_t)s->cells + 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t h = s->hash[i];
        uint32_t p = s->cell_first[h] + fill[h]++;
        s->sorted_idx[p] = i;
    }
    free(fill);
    for (uint32_t p = 0; p < n; ++p) {
        uint32_t i = s->sorted_idx[p];
        for (int d = 0; d < 4; ++d) {
            s->sx[4 * p + d] = s->x[4 * i + d];
            s->sx32[4 * p + d] = (float)R_VAL(s->x[4 * i + d]);
        }
        s->sphase[p] = s->phase[i];
        s->srho0[p] = s->rho0[i];
    }
    s->grid_valid = 1;
}

/* ---- PBF */

typedef struct {
    const orc_system *s;
    uint32_t i, nb, cap;
    const float *pi32;
    uint32_t *list;   /* neighbour sorted indices, in visiting order */
} nb_ctx;

static int fluid_visit(void *vctx, uint32_t j) {
    nb_ctx *c = (nb_ctx *)vctx;
    if (j == c->i) return 0;
    /* PBD_FLAG_SKIP_FIXED_NEIGHBORS: fixed particles are no neighbours
     * (totalfluidconstraint.cpp:59) */
    if ((c->s->p.flags & PBD_FLAG_SKIP_FIXED_NEIGHBORS) && c->s->sx32[4 * j + 3] == 0.f) return 0;
    float d2 = dist2f(c->pi32, c->s->sx32 + 4 * j);
    if (d2 < c->s->h2f) {
        if (c->nb >= c->s->p.max_neighbors) return 1;
        c->list[c->nb++] = j;
    }
    return 0;
}

static uint32_t fluid_neighbors(const orc_system *s, uint32_t i, uint32_t *list) {
    nb_ctx c = {s, i, 0, s->p.max_neighbors, s->sx32 + 4 * i, list};
    int g[3];
    grid_cell(s, s->sx32 + 4 * i, g);
    for_each_candidate(s, g, s->fluid_rad, fluid_visit, &c);
    return c.nb;
}

/* Neighbours of gas particle i: particles with w > 0 (gasconstraint.cpp:46)
 * closer than h, in visiting order, at most max_neighbors. */
static int gas_visit(void *vctx, uint32_t j) {
    nb_ctx *c = (nb_ctx *)vctx;
    if (j == c->i) return 0;
    float d2 = dist2f(c->pi32, c->s->sx32 + 4 * j);
    if (d2 < c->s->h2f && c->s->sx32[4 * j + 3] > 0.f) {
        if (c->nb >= c->s->p.max_neighbors) return 1;
        c->list[c->nb++] = j;
    }
    return 0;
}

static uint32_t gas_neighbors(const orc_system *s, uint32_t i, uint32_t *list) {
    nb_ctx c = {s, i, 0, s->p.max_neighbors, s->sx32 + 4 * i, list};
    int g[3];
    grid_cell(s, s->sx32 + 4 * i, g);
    for_each_candidate(s, g, s->fluid_rad, gas_visit, &c);
    return c.nb;
}

/* The lambda half of GasConstraint::project (gasconstraint.cpp:34-83):
 * rho = sum poly6 m_j s_j + poly6(0) m_i (s_j = S_SOLID for solid-like
 * neighbours), gradients unweighted, lambda = -(rho / rho0 - 1) / (denom +
 * relaxation); an open gas adds v' (1 - rho / rho0) (-drag) to the force
 * (gasconstraint.cpp:80). */
static void gas_lambda(orc_system *s, uint32_t i, uint32_t *list) {
    uint32_t nb = gas_neighbors(s, i, list);
    s->nb_fluid[s->sorted_idx[i]] = nb;
    const real *pi = s->sx + 4 * i;
    const double rho0 = s->srho0[i];
    const double h = s->p.kernel_radius, h2 = h * h;
    real ro = 0, denom = 0, grad[3] = {0, 0, 0};
    for (uint32_t k = 0; k < nb; ++k) {
        const real *pj = s->sx + 4 * list[k];
        real r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
        real r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        real rlen = sqrt(r2);
        real hm2 = h2 - r2, hm = h - rlen;
        const double sw = s->sphase[list[k]] >= PBD_PHASE_CLOTH ? (double)s->p.gas_solid_density_weight : 1.0;
        ro += sw * s->poly6 * hm2 * hm2 * hm2 / pj[3];
        real sg[3] = {0, 0, 0};
        if (dist2f(s->sx32 + 4 * i, s->sx32 + 4 * list[k]) >= K_MIN_SPIKY2)
            for (int d = 0; d < 3; ++d) sg[d] = r[d] / rlen * (-s->spiky * hm * hm) / rho0;
        for (int d = 0; d < 3; ++d) {
            grad[d] -= sg[d];
            denom += sg[d] * sg[d];
        }
    }
    ro += s->poly6_self / pi[3];
    denom += grad[0] * grad[0] + grad[1] * grad[1] + grad[2] * grad[2];
    const real ratio = ro / rho0;
    s->glambda[i] = -(ratio - 1.0) / (denom + s->relax);
    s->lambda[i] = 0.0;
    const uint32_t o = s->sorted_idx[i];
    if (s->gas_open[o])
        for (int d = 0; d < 3; ++d) s->force[4 * o + d] += s->v[4 * o + d] * ((1.0 - ratio) * -(double)s->p.gas_drag);
}

/* findLambdasD (integration_kernel.cuh:521-593). */
static void compute_lambdas(orc_system *s) {
    const uint32_t n = s->n;
    const int nb_mass = (s->p.flags & PBD_FLAG_DENSITY_NEIGHBOR_MASS) != 0;
    set_threads();
#pragma omp parallel
    {
        uint32_t *list = (uint32_t *)malloc(s->p.max_neighbors * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1024)
        for (long long ii = 0; ii < (long long)n; ++ii) {
            uint32_t i = (uint32_t)ii;
            if (s->sphase[i] == PBD_PHASE_GAS) {
                gas_lambda(s, i, list);
                continue;
            }
            if (s->sphase[i] != PBD_PHASE_FLUID) {
                s->lambda[i] = 0.0;
                continue;
            }
            uint32_t nb = fluid_neighbors(s, i, list);
            s->nb_fluid[s->sorted_idx[i]] = nb;
            const real *pi = s->sx + 4 * i;
            const real w = pi[3];
            const double rho0 = s->srho0[i];
            const double h = s->p.kernel_radius, h2 = h * h;
            real ro = 0, denom = 0, grad[3] = {0, 0, 0};
            for (uint32_t k = 0; k < nb; ++k) {
                const real *pj = s->sx + 4 * list[k];
                real r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
                real r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
                real rlen = sqrt(r2);
                real hm2 = h2 - r2, hm = h - rlen;
                real wpoly = s->poly6 * hm2 * hm2 * hm2;
                /* a solid-like neighbour's weight in the density and in the
                 * particle's own gradient (totalfluidconstraint.cpp:66-68,
                 * 154); the pair gradient itself is not weighted */
                const double sw = s->sphase[list[k]] >= PBD_PHASE_CLOTH ? (double)s->p.solid_density_weight : 1.0;
                if (nb_mass) ro += pj[3] > 0 ? sw * wpoly / pj[3] : 0.0;
                else ro += sw * wpoly / w;
                real sg[3] = {0, 0, 0};
                /* the cut-off is decided on the FP32 length, as the kernel does */
                if (dist2f(s->sx32 + 4 * i, s->sx32 + 4 * list[k]) >= K_MIN_SPIKY2)
                    for (int d = 0; d < 3; ++d) sg[d] = r[d] / rlen * (-s->spiky * hm * hm);
                for (int d = 0; d < 3; ++d) {
                    sg[d] /= rho0;
                    grad[d] -= sw * sg[d];
                    denom += sg[d] * sg[d];
                }
            }
            ro += s->poly6_self / w;
            denom += grad[0] * grad[0] + grad[1] * grad[1] + grad[2] * grad[2];
            s->lambda[i] = -(ro / rho0 - 1.0) / (denom + s->relax);
        }
        free(list);
    }
}

static real scorr_pow(const orc_system *s, real ratio) { return pow(ratio, (double)s->p.scorr_n); }

/* solveFluidsD (integration_kernel.cuh:596-642). */
static void fluid_delta(const orc_system *s, uint32_t i, uint32_t *list, real out[3]) {
    uint32_t nb = fluid_neighbors(s, i, list);
    const real *pi = s->sx + 4 * i;
    const double h = s->p.kernel_radius, h2 = h * h;
    real delta[3] = {0, 0, 0};
    for (uint32_t k = 0; k < nb; ++k) {
        uint32_t j = list[k];
        const real *pj = s->sx + 4 * j;
        real r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
        real r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        real rlen = sqrt(r2);
        real hm2 = h2 - r2, hm = h - rlen;
        real sc = -s->spiky * hm * hm;
        real sg[3];
        if (dist2f(s->sx32 + 4 * i, s->sx32 + 4 * j) < K_MIN_SPIKY2) {
            sg[0] = 0; sg[1] = K_EPS * sc; sg[2] = 0;
        } else {
            for (int d = 0; d < 3; ++d) sg[d] = r[d] / rlen * sc;
        }
        real ratio = s->poly6 * hm2 * hm2 * hm2 * s->scorr_inv_ref;
        real corr = -s->scorr_k * scorr_pow(s, ratio);
        real coef = s->lambda[i] + s->lambda[j] + corr;
        for (int d = 0; d < 3; ++d) delta[d] += coef * sg[d];
    }
    /* rho0 + n (integration_kernel.cuh:640), rho0, or rho0 (n + 1): the
     * CPU reference's delta / p0 / (neighbours incl. self + counts, the
     * counts zero for fluid; totalfluidconstraint.cpp:108,114) */
    double div = (s->p.flags & PBD_FLAG_DELTA_OVER_COUNT) ? s->srho0[i] * (double)(nb + 1)
                 : (s->p.flags & PBD_FLAG_DELTA_OVER_RHO0) ? s->srho0[i]
                                                            : s->srho0[i] + (double)nb;
    for (int d = 0; d < 3; ++d) out[d] = delta[d] / div;
}

/* The delta half of GasConstraint::project (gasconstraint.cpp:86-121):
 * sum (lambda_i + lambda_j + s_corr) spikyGrad / rho0 / (neighbours + 1),
 * lambda_j of gas neighbours only (the reference's per-constraint lambdas),
 * s_corr = -K_P (poly6(r) / poly6(DQ_P h))^n, spikyGrad zero below the FP32
 * length cut-off.  The vorticity term goes to the force: f += sum (-|w| r_y,
 * |w| r_x, 0) poly6(r), w = spikyGrad evaluated at |r|^2 (the reference
 * passes glm::dot(r, r)) times v'_j componentwise; zero for |r|^2 >= h. */
static void gas_delta(orc_system *s, uint32_t i, uint32_t *list, real out[3]) {
    uint32_t nb = gas_neighbors(s, i, list);
    const real *pi = s->sx + 4 * i;
    const double h = s->p.kernel_radius, h2 = h * h;
    real delta[3] = {0, 0, 0}, fv[2] = {0, 0};
    for (uint32_t k = 0; k < nb; ++k) {
        uint32_t j = list[k];
        const real *pj = s->sx + 4 * j;
        real r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
        real r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        real rlen = sqrt(r2);
        real hm2 = h2 - r2, hm = h - rlen;
        real wp = s->poly6 * hm2 * hm2 * hm2;
        const int far = dist2f(s->sx32 + 4 * i, s->sx32 + 4 * j) >= K_MIN_SPIKY2;
        real sg[3] = {0, 0, 0};
        if (far)
            for (int d = 0; d < 3; ++d) sg[d] = r[d] / rlen * (-s->spiky * hm * hm);
        real corr = -s->gas_scorr_k * scorr_pow(s, wp * s->gas_scorr_inv_ref);
        real lj = s->sphase[j] == PBD_PHASE_GAS ? s->glambda[j] : (real)0.0;
        real coef = s->glambda[i] + lj + corr;
        for (int d = 0; d < 3; ++d) delta[d] += coef * sg[d];
        if (far && r2 < h) {
            const real *vj = s->v + 4 * s->sorted_idx[j];
            real hq = h - r2;
            real w[3];
            for (int d = 0; d < 3; ++d) w[d] = r[d] / rlen * (-s->spiky * hq * hq) * vj[d];
            real wl = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            fv[0] -= wl * r[1] * wp;
            fv[1] += wl * r[0] * wp;
        }
    }
    const uint32_t o = s->sorted_idx[i];
    s->force[4 * o] += fv[0];
    s->force[4 * o + 1] += fv[1];
    const double div = s->srho0[i] * (double)(nb + 1);
    for (int d = 0; d < 3; ++d) out[d] = delta[d] / div;
}

/* ---- contacts */

typedef struct {
    const orc_system *s;
    uint32_t i, nb;
    int ph;
    uint32_t *list;
} ct_ctx;

static int contact_visit(void *vctx, uint32_t j) {
    ct_ctx *c = (ct_ctx *)vctx;
    if (j == c->i) return 0;
    int phj = c->s->sphase[j];
    if (c->ph > PBD_PHASE_SOLID && c->ph == phj) return 0;
    const int cpu = (c->s->p.flags & PBD_FLAG_CPU_CONTACTS) != 0;
    /* PBD_FLAG_CPU_CONTACTS: never two fixed particles (simulation.cpp:174) */
    if (cpu && c->s->sx32[4 * c->i + 3] == 0.f && c->s->sx32[4 * j + 3] == 0.f) return 0;
    if (dist2f(c->s->sx32 + 4 * c->i, c->s->sx32 + 4 * j) < (cpu ? c->s->cpu_c2f : c->s->collide2f)) {
        if (c->nb >= c->s->p.max_neighbors) return 1;
        c->list[c->nb++] = j;
    }
    return 0;
}

static real scaled_w(real w, real y) { return w != 0.0 ? 1.0 / ((1.0 / w) * exp(-y)) : w; }

#define CPU_EPS 0.0001 /* EPSILON, cpu/src/includes.h:34 */

static void quat_rotate(const real q[4], const double v[3], real out[3]) {
    real t[3] = {2.0 * (q[1] * v[2] - q[2] * v[1]), 2.0 * (q[2] * v[0] - q[0] * v[2]), 2.0 * (q[0] * v[1] - q[1] * v[0])};
    out[0] = v[0] + q[3] * t[0] + (q[1] * t[2] - q[2] * t[1]);
    out[1] = v[1] + q[3] * t[1] + (q[2] * t[0] - q[0] * t[2]);
    out[2] = v[2] + q[3] * t[2] + (q[0] * t[1] - q[1] * t[0]);
}

/* The correction and friction of RigidContactConstraint::project
 * (rigidcontactconstraint.cpp:58-95) for the ordered pair (1, 2) with depth
 * d along n, as seen by particle 1 (first) or 2: d n shared by the
 * height-scaled inverse masses tmass = w e^y (Particle::scaleMass, at the
 * start-of-step heights) and averaged over cnt (this particle's count, for
 * both ends); then the tangential relative displacement since the step's
 * start removed if below mu_s d (static), else cut by min(mu_k d / |dpt|,
 * 1).  Adds to out. */
static void rigid_contact_apply(const orc_system *s, int first, const real *x1, const real *x2, const real *p1,
                                const real *p2, real d, const real n[3], double cnt, real out[3]) {
    const double w1 = R_VAL(x1[3]), w2 = R_VAL(x2[3]);
    real t1 = w1 * exp(p1[1]), t2 = w2 * exp(p2[1]);
    real tsum = t1 + t2;
    if (!(R_VAL(tsum) > 0.0)) return;
    real a1 = t1 / tsum, a2 = t2 / tsum, dp1[3], dp2[3];
    for (int k = 0; k < 3; ++k) {
        dp1[k] = -a1 * d * n[k] / cnt;
        dp2[k] = a2 * d * n[k] / cnt;
        out[k] += first ? dp1[k] : dp2[k];
    }
    real nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    real nf[3] = {n[0] / nl, n[1] / nl, n[2] / nl}, dpf[3], dpt[3];
    for (int k = 0; k < 3; ++k) dpf[k] = (x1[k] + dp1[k] - p1[k]) - (x2[k] + dp2[k] - p2[k]);
    real dn = dpf[0] * nf[0] + dpf[1] * nf[1] + dpf[2] * nf[2];
    for (int k = 0; k < 3; ++k) dpt[k] = dpf[k] - dn * nf[k];
    real ldpt = sqrt(dpt[0] * dpt[0] + dpt[1] * dpt[1] + dpt[2] * dpt[2]);
    if (ldpt < CPU_EPS) return;
    real f = 1.0;
    if (!(ldpt < (double)s->p.contact_static_friction * d)) {
        f = (double)s->p.contact_kinetic_friction * d / ldpt;
        if (f > 1.0) f = 1.0;
    }
    for (int k = 0; k < 3; ++k) out[k] += (first ? -a1 : a2) * dpt[k] * f;
}

/* RigidContactConstraint::project (rigidcontactconstraint.cpp:30-96) for a
 * pair of particles with signed-distance data, as seen by particle `self`
 * (original index) against `other`: the pair is ordered by original index;
 * depth and normal from the particle nearer its surface, replaced below
 * one diameter + EPSILON by initBoundary (:13-27); correction and friction
 * shared by the height-scaled inverse masses tmass = w e^y at the
 * start-of-step heights (Particle::scaleMass); averaged over `cnt` (this
 * particle's contact count, for both ends).  Adds to out. */
static void sdf_contact(const orc_system *s, uint32_t self, uint32_t other, const real *xs, const real *xo,
                        const real *ps, const real *po, double cnt, real out[3]) {
    const int first = self < other;
    const uint32_t o1 = first ? self : other, o2 = first ? other : self;
    const real *x1 = first ? xs : xo, *x2 = first ? xo : xs, *p1 = first ? ps : po, *p2 = first ? po : ps;
    const double *s1 = s->sdf + 4 * o1, *s2 = s->sdf + 4 * o2;
    real n1[3], n2[3], n[3];
    quat_rotate(s->bquat + 4 * s->body_of[o1], s1, n1);
    quat_rotate(s->bquat + 4 * s->body_of[o2], s2, n2);
    real d;
    if (s1[3] < s2[3]) {
        d = s1[3];
        for (int k = 0; k < 3; ++k) n[k] = n1[k];
    } else {
        d = s2[3];
        for (int k = 0; k < 3; ++k) n[k] = -n2[k];
    }
    const double diam = 2.0 * (double)s->p.particle_radius;
    if (d < diam + CPU_EPS) {
        real x12[3] = {x1[0] - x2[0], x1[1] - x2[1], x1[2] - x2[2]};
        real len = sqrt(x12[0] * x12[0] + x12[1] * x12[1] + x12[2] * x12[2]);
        d = diam - len;
        if (d < CPU_EPS) return;
        if (len > CPU_EPS) {
            for (int k = 0; k < 3; ++k) x12[k] = x12[k] / len;
        } else {
            x12[0] = 0.0; x12[1] = 1.0; x12[2] = 0.0;
        }
        real dp = x12[0] * n[0] + x12[1] * n[1] + x12[2] * n[2];
        for (int k = 0; k < 3; ++k) n[k] = dp < 0.0 ? x12[k] - 2.0 * dp * n[k] : x12[k];
    }
    rigid_contact_apply(s, first, x1, x2, p1, p2, d, n, cnt, out);
}

/* PBD_FLAG_CPU_CONTACTS, two solid-like particles without signed-distance
 * data: RigidContactConstraint::project's plain branch
 * (rigidcontactconstraint.cpp:35-41): d = diameter - |x2 - x1|, n = (x2 -
 * x1) / |x2 - x1| for the pair ordered by original index; correction and
 * friction as rigid_contact_apply.  Adds to out. */
static void cpu_pair_contact(const orc_system *s, uint32_t self, uint32_t other, const real *xs, const real *xo,
                             const real *ps, const real *po, double cnt, real out[3]) {
    const int first = self < other;
    const real *x1 = first ? xs : xo, *x2 = first ? xo : xs;
    real x12[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
    real len = sqrt(x12[0] * x12[0] + x12[1] * x12[1] + x12[2] * x12[2]);
    real d = 2.0 * (double)s->p.particle_radius - len;
    if (d < CPU_EPS) return;
    real n[3] = {x12[0] / len, x12[1] / len, x12[2] / len};
    rigid_contact_apply(s, first, x1, x2, first ? ps : po, first ? po : ps, d, n, cnt, out);
}

/* PBD_FLAG_CPU_CONTACTS, a solid-like particle touching a fluid or gas one:
 * ContactConstraint::project (contactconstraint.cpp:13-42) for this end:
 * the overlap shared by the height-scaled inverse masses, averaged over the
 * count, no friction (the fluid end is not moved: fluid takes no part in
 * the contact pass).  Adds to out. */
static void cpu_fluid_contact(const orc_system *s, const real *xs, const real *xo, const real *ps, const real *po,
                              double cnt, real out[3]) {
    real diff[3] = {xs[0] - xo[0], xs[1] - xo[1], xs[2] - xo[2]};
    real dist = sqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
    real mag = dist - 2.0 * (double)s->p.particle_radius;
    if (R_VAL(mag) > 0.0 || R_VAL(dist) == 0.0) return;
    real ts = xs[3] * exp(ps[1]), to = xo[3] * exp(po[1]);
    real tsum = ts + to;
    if (!(R_VAL(tsum) > 0.0)) return;
    for (int k = 0; k < 3; ++k) out[k] += -(ts / tsum) * mag * diff[k] / (dist * cnt);
}

/* Walls a particle touches (the CPU reference's boundary detection,
 * simulation.cpp:202-224: per axis the lower wall, else the upper). */
static int cpu_wall_count(const orc_system *s, const real *e) {
    const double r = s->p.particle_radius;
    int k = 0;
    k += (e[0] < s->p.box_min[0] + r || e[0] > s->p.box_max[0] - r);
    k += (e[1] < s->p.box_min[1] + r || e[1] > s->p.box_max[1] - r);
    if (!(s->p.flags & PBD_FLAG_TWOD)) k += (e[2] < s->p.box_min[2] + r || e[2] > s->p.box_max[2] - r);
    return k;
}

/* collideD + collideCell (integration_kernel.cuh:303-462).  Pairs with zero
 * total inverse mass or zero separation are skipped (NaN in the reference). */
static double contact_delta(const orc_system *s, uint32_t i, uint32_t *list, real out[3]) {
    ct_ctx c = {s, i, 0, s->sphase[i], list};
    int g[3];
    grid_cell(s, s->sx32 + 4 * i, g);
    for_each_candidate(s, g, 1, contact_visit, &c);
    s->nb_contact[s->sorted_idx[i]] = c.nb;
    out[0] = out[1] = out[2] = 0;
    const int cpu = (s->p.flags & PBD_FLAG_CPU_CONTACTS) != 0;
    const real *pi = s->sx + 4 * i;
    /* the CPU reference averages over every constraint of the group:
     * contacts and walls (updateCounts) */
    const double fnb = (double)c.nb + (cpu ? (double)cpu_wall_count(s, pi) : 0.0);
    if (!c.nb) return fnb;
    const real w = pi[3], sw = scaled_w(w, pi[1]);
    const real *prev = s->x_old + 4 * s->sorted_idx[i];
    const int ph = s->sphase[i];
    const double cdist = (double)s->collidef;
    const uint32_t oi = s->sorted_idx[i];
    const int sdf_i = s->any_sdf && ph >= PBD_PHASE_SOLID && s->sdf[4 * oi + 3] >= 0.0;
    for (uint32_t k = 0; k < c.nb; ++k) {
        uint32_t j = list[k];
        const real *pj = s->sx + 4 * j;
        int phj = s->sphase[j];
        if (sdf_i && phj >= PBD_PHASE_SOLID && s->sdf[4 * s->sorted_idx[j] + 3] >= 0.0) {
            const uint32_t oj = s->sorted_idx[j];
            sdf_contact(s, oi, oj, pi, pj, prev, s->x_old + 4 * oj, fnb, out);
            continue;
        }
        if (cpu) {
            const uint32_t oj = s->sorted_idx[j];
            if (phj >= PBD_PHASE_CLOTH) cpu_pair_contact(s, oi, oj, pi, pj, prev, s->x_old + 4 * oj, fnb, out);
            else cpu_fluid_contact(s, pi, pj, prev, s->x_old + 4 * oj, fnb, out);
            continue;
        }
        real diff[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
        real dist = sqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
        real mag = dist - cdist;
        real colw = w, colw2 = pj[3];
        if (ph >= PBD_PHASE_SOLID && phj >= PBD_PHASE_SOLID) {
            colw = sw;
            colw2 = scaled_w(pj[3], pi[1]);
        }
        real wsum = colw + colw2;
        if (wsum == 0.0 || dist == 0.0) continue;
        real scale = mag / wsum, dp[3], dp1[3], dp2[3];
        for (int d = 0; d < 3; ++d) {
            dp[d] = diff[d] * (scale / dist);
            dp1[d] = -colw * dp[d] / fnb;
            dp2[d] = colw2 * dp[d] / fnb;
            out[d] += dp1[d];
        }
        if (ph < PBD_PHASE_SOLID || phj < PBD_PHASE_SOLID) continue;
        const real *prev2 = s->x_old + 4 * s->sorted_idx[j];
        real nf[3] = {diff[0] / dist, diff[1] / dist, diff[2] / dist};
        real dprel[3], dpt[3];
        for (int d = 0; d < 3; ++d) dprel[d] = (pi[d] + dp1[d] - prev[d]) - (prev[d] + dp2[d] - prev2[d]);
        real dn = dprel[0] * nf[0] + dprel[1] * nf[1] + dprel[2] * nf[2];
        for (int d = 0; d < 3; ++d) dpt[d] = dprel[d] - dn * nf[d];
        real ldpt = sqrt(dpt[0] * dpt[0] + dpt[1] * dpt[1] + dpt[2] * dpt[2]);
        if (ldpt < K_EPS) continue;
        if (ldpt < (double)s->p.contact_static_friction * dist) {
            for (int d = 0; d < 3; ++d) out[d] -= dpt[d] * colw / wsum;
        } else {
            real f = fmin((double)s->p.contact_kinetic_friction * dist / ldpt, 1.0);
            for (int d = 0; d < 3; ++d) out[d] -= dpt[d] * f;
        }
    }
    return fnb;
}

/* PBD_FLAG_CPU_CONTACTS: BoundaryConstraint::project (boundaryconstraint.cpp:
 * 14-93) for each wall passed, x then y (then z): back to the wall + r (the
 * reference's fluid jitter left out), then the tangential part of (e -
 * p_old) / count removed if below sqrt(mu_s) r, else cut by min(sqrt(mu_k)
 * r / |dpt|, 1). */
static void cpu_boundaries(const orc_system *s, real e[3], const real *xold, double count) {
    const double r = s->p.particle_radius;
    const int twod = (s->p.flags & PBD_FLAG_TWOD) != 0;
    const int axes = twod ? 2 : 3;
    for (int a = 0; a < axes; ++a) {
        const double lo = s->p.box_min[a], hi = s->p.box_max[a];
        double sgn;
        if (e[a] < lo + r) {
            e[a] = lo + r;
            sgn = 1.0;
        } else if (e[a] > hi - r) {
            e[a] = hi - r;
            sgn = -1.0;
        } else {
            continue;
        }
        real pold[3] = {xold[0], xold[1], twod ? (real)s->p.twod_z : xold[2]};
        real dp[3], nrm[3] = {0, 0, 0};
        nrm[a] = sgn;
        for (int k = 0; k < 3; ++k) dp[k] = (e[k] - pold[k]) / count;
        real dn = dp[a] * sgn;
        real dpt[3] = {dp[0] - dn * nrm[0], dp[1] - dn * nrm[1], dp[2] - dn * nrm[2]};
        real ldpt = sqrt(dpt[0] * dpt[0] + dpt[1] * dpt[1] + dpt[2] * dpt[2]);
        if (ldpt < CPU_EPS) continue;
        if (ldpt < s->ws * r) {
            for (int k = 0; k < 3; ++k) e[k] -= dpt[k];
        } else {
            real f = fmin(s->wk * r / ldpt, 1.0);
            for (int k = 0; k < 3; ++k) e[k] -= dpt[k] * f;
        }
    }
    if (twod) e[2] = s->p.twod_z;
}

/* collide_world_functor (integration_kernel.cuh:57-157); with
 * PBD_FLAG_CPU_CONTACTS the CPU reference's boundaries, averaged over
 * `count` (contacts and walls of a contact particle; 0 = walls only). */
static void world_collide(const orc_system *s, real e[3], int phase, const real *xold, double count) {
    if (s->p.flags & PBD_FLAG_CPU_CONTACTS) {
        if (count < 1.0) count = (double)cpu_wall_count(s, e);
        if (count < 1.0) {
            if (s->p.flags & PBD_FLAG_TWOD) e[2] = s->p.twod_z;
            return;
        }
        cpu_boundaries(s, e, xold, count);
        return;
    }
    const double r = s->p.particle_radius, d = r;
    const double *bmin = NULL;
    double lo[3] = {s->p.box_min[0], s->p.box_min[1], s->p.box_min[2]};
    double hi[3] = {s->p.box_max[0], s->p.box_max[1], s->p.box_max[2]};
    const int twod = (s->p.flags & PBD_FLAG_TWOD) != 0;
    (void)bmin;
    double eps = phase < PBD_PHASE_SOLID ? d * 0.01 : 0.0;
    double n[3] = {0, 0, 0};
    if (e[1] < lo[1] + r) { e[1] = lo[1] + r + s->rands[5] * eps; n[1] += 1; }
    eps = d * 0.01;
    if (e[0] > hi[0] - r) { e[0] = hi[0] - (r + s->rands[0] * eps); n[0] -= 1; }
    if (e[0] < lo[0] + r) { e[0] = lo[0] + (r + s->rands[1] * eps); n[0] += 1; }
    if (e[1] > hi[1] - r) { e[1] = hi[1] - (r + s->rands[2] * eps); n[1] -= 1; }
    if (!twod) {
        if (e[2] > hi[2] - r) { e[2] = hi[2] - (r + s->rands[3] * eps); n[2] -= 1; }
        if (e[2] < lo[2] + r) { e[2] = lo[2] + (r + s->rands[4] * eps); n[2] += 1; }
    } else {
        e[2] = s->p.twod_z;
    }
    if (sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) < K_EPS || phase < PBD_PHASE_CLOTH) return;
    real pos[3] = {xold[0], xold[1], twod ? (real)s->p.twod_z : xold[2]};
    real dp[3] = {e[0] - pos[0], e[1] - pos[1], e[2] - pos[2]};
    real dn = dp[0] * n[0] + dp[1] * n[1] + dp[2] * n[2];
    real dpt[3] = {dp[0] - dn * n[0], dp[1] - dn * n[1], dp[2] - dn * n[2]};
    real ldpt = sqrt(dpt[0] * dpt[0] + dpt[1] * dpt[1] + dpt[2] * dpt[2]);
    if (ldpt < K_EPS) return;
    if (ldpt < s->ws * d) {
        for (int k = 0; k < 3; ++k) e[k] -= dpt[k];
    } else {
        real f = fmin(s->wk * d / ldpt, 1.0);
        for (int k = 0; k < 3; ++k) e[k] -= dpt[k] * f;
    }
}

enum { DO_CONTACT = 1, DO_FLUID = 2, DO_WORLD = 4 };

/* The reference's collide, solveFluids (delta) and collideWorld: disjoint
 * particle sets reading the sorted start-of-iteration positions, so they
 * can run as one pass (same order of effects as the CUDA k_solve). */
static void solve_pass(orc_system *s, int mask) {
    const uint32_t n = s->n;
    if (mask & DO_FLUID) compute_lambdas(s);
    real *out = (real *)malloc(4ull * (n ? n : 1) * sizeof(real));
    unsigned char *touched = (unsigned char *)calloc(n ? n : 1, 1);
    set_threads();
#pragma omp parallel
    {
        uint32_t *list = (uint32_t *)malloc(s->p.max_neighbors * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1024)
        for (long long ii = 0; ii < (long long)n; ++ii) {
            uint32_t i = (uint32_t)ii, o = s->sorted_idx[i];
            int ph = s->sphase[i];
            real np[3] = {s->sx[4 * i], s->sx[4 * i + 1], s->sx[4 * i + 2]}, dd[3];
            int t = 0;
            double count = 0.0;
            if ((mask & DO_FLUID) && ph == PBD_PHASE_FLUID) {
                fluid_delta(s, i, list, dd);
                for (int d = 0; d < 3; ++d) np[d] += dd[d];
                t = 1;
            } else if ((mask & DO_FLUID) && ph == PBD_PHASE_GAS) {
                gas_delta(s, i, list, dd);
                for (int d = 0; d < 3; ++d) np[d] += dd[d];
                t = 1;
            } else if ((mask & DO_CONTACT) && ph >= PBD_PHASE_CLOTH) {
                count = contact_delta(s, i, list, dd);
                for (int d = 0; d < 3; ++d) np[d] += dd[d];
                t = 1;
            }
            if (mask & DO_WORLD) {
                if (!t)
                    for (int d = 0; d < 3; ++d) np[d] = s->x[4 * o + d];
                world_collide(s, np, ph, s->x_old + 4 * o, count);
                t = 1;
            }
            if (t) {
                touched[i] = 1;
                for (int d = 0; d < 3; ++d) out[4 * i + d] = np[d];
            }
        }
        free(list);
    }
    for (uint32_t i = 0; i < n; ++i)
        if (touched[i]) {
            uint32_t o = s->sorted_idx[i];
            for (int d = 0; d < 3; ++d) s->x[4 * o + d] = out[4 * i + d];
        }
    free(out);
    free(touched);
}

void orc_collide(orc_system *s) { solve_pass(s, DO_CONTACT); }
void orc_solve_fluids(orc_system *s) { solve_pass(s, DO_FLUID); }
void orc_collide_world(orc_system *s) { solve_pass(s, DO_WORLD); }

/* ---- distance constraints and pins */

/* delta_computing_functor / reduce_by_key / distance_constraint_functor
 * (solver_kernel.cuh:27-72,155-163; solver.cu:196-231): every constraint
 * adds +-n (rest - d) / 2 (times stiffness; PBD_FLAG_DISTANCE_MASS_WEIGHTED:
 * w_k / (w_a + w_b) instead of 1/2) to its endpoints, summed per particle
 * and divided by the particle's constraint count (distance + point,
 * updateOccurences solver.cu:72-106).  Applied to the right particle (the
 * reference applied segment k to particle k, solver.cu:227-230). */
void orc_solve_distance_constraints(orc_system *s) {
    const uint32_t n = s->n;
    if (!s->m) return;
    real *acc = (real *)calloc(3ull * n, sizeof(real));
    uint32_t *occ = (uint32_t *)calloc(n, sizeof(uint32_t));
    for (uint32_t c = 0; c < s->m; ++c) {
        ++occ[s->da[c]];
        ++occ[s->db[c]];
    }
    for (uint32_t k = 0; k < s->npin; ++k) ++occ[s->pin_idx[k]];
    const int mw = (s->p.flags & PBD_FLAG_DISTANCE_MASS_WEIGHTED) != 0;
    for (uint32_t c = 0; c < s->m; ++c) {
        const real *a = s->x + 4 * s->da[c], *b = s->x + 4 * s->db[c];
        real rel[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
        real dist = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
        if (!(dist > K_MIN_DIST)) continue;
        real ma, mb;
        if (mw) {
            real ws = a[3] + b[3];
            ma = ws > 0 ? (s->drest[c] - dist) * (a[3] / ws) : 0.0;
            mb = ws > 0 ? (s->drest[c] - dist) * (b[3] / ws) : 0.0;
        } else {
            ma = mb = (s->drest[c] - dist) * 0.5;
        }
        ma *= s->dstiff[c];
        mb *= s->dstiff[c];
        for (int d = 0; d < 3; ++d) {
            acc[3 * s->da[c] + d] += rel[d] / dist * ma;
            acc[3 * s->db[c] + d] -= rel[d] / dist * mb;
        }
    }
    for (uint32_t k = 0; k < n; ++k)
        if (occ[k])
            for (int d = 0; d < 3; ++d) s->x[4 * k + d] += acc[3 * k + d] / (double)occ[k];
    free(acc);
    free(occ);
}

/* point_constraint_functor (solver_kernel.cuh:10-25); the last pin on a
 * particle wins. */
void orc_solve_point_constraints(orc_system *s) {
    for (uint32_t k = 0; k < s->npin; ++k)
        for (int d = 0; d < 3; ++d) s->x[4 * s->pin_idx[k] + d] = s->pin_pts[3 * k + d];
}

/* ---- shape matching */

static void quat_to_mat(const real q[4], real R[3][3]) {
    real x = q[0], y = q[1], z = q[2], w = q[3];
    R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - w * z);     R[0][2] = 2 * (x * z + w * y);
    R[1][0] = 2 * (x * y + w * z);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - w * x);
    R[2][0] = 2 * (x * z - w * y);     R[2][1] = 2 * (y * z + w * x);     R[2][2] = 1 - 2 * (x * x + y * y);
}

/* Rotation extraction of Mueller, Bender, Chentanez, Macklin, "A Robust
 * Method to Extract the Rotational Part of Deformations" (MIG 2016). */
static void extract_rotation(const real A[3][3], real q[4], int iters) {
    for (int it = 0; it < iters; ++it) {
        real R[3][3];
        quat_to_mat(q, R);
        real o[3] = {0, 0, 0}, dsum = 0;
        for (int c = 0; c < 3; ++c) {
            real rx = R[0][c], ry = R[1][c], rz = R[2][c];
            real ax = A[0][c], ay = A[1][c], az = A[2][c];
            o[0] += ry * az - rz * ay;
            o[1] += rz * ax - rx * az;
            o[2] += rx * ay - ry * ax;
            dsum += rx * ax + ry * ay + rz * az;
        }
        real inv = 1.0 / (fabs(dsum) + 1.0e-9);
        for (int k = 0; k < 3; ++k) o[k] *= inv;
        real wl = sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        if (wl < 1.0e-9) break;
        real sh = sin(0.5 * wl) / wl, ch = cos(0.5 * wl);
        real d[4] = {o[0] * sh, o[1] * sh, o[2] * sh, ch};
        real r[4];
        r[3] = d[3] * q[3] - d[0] * q[0] - d[1] * q[1] - d[2] * q[2];
        r[0] = d[3] * q[0] + d[0] * q[3] + d[1] * q[2] - d[2] * q[1];
        r[1] = d[3] * q[1] - d[0] * q[2] + d[1] * q[3] + d[2] * q[0];
        r[2] = d[3] * q[2] + d[0] * q[1] - d[1] * q[0] + d[2] * q[3];
        real qn = 1.0 / sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
        for (int k = 0; k < 4; ++k) q[k] = r[k] * qn;
    }
}

/* Shape matching (Mueller, Heidelberger, Teschner, Gross 2005) in 3-D; the
 * reference's 2-D counterpart is TotalShapeConstraint::project
 * (cpu/src/constraint/totalshapeconstraint.cpp:14-24). */
void orc_solve_shapes(orc_system *s) {
    for (uint32_t b = 0; b < s->nb; ++b) {
        uint32_t f = s->bfirst[b], cnt = s->bcount[b];
        real c[3] = {0, 0, 0};
        double msum = 0;
        for (uint32_t k = f; k < f + cnt; ++k) {
            double m = s->brest[4 * k + 3];
            for (int d = 0; d < 3; ++d) c[d] += m * s->x[4 * k + d];
            msum += m;
        }
        for (int d = 0; d < 3; ++d) c[d] /= msum;
        real A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (uint32_t k = f; k < f + cnt; ++k) {
            const double *q = s->brest + 4 * k;
            for (int r = 0; r < 3; ++r)
                for (int cc = 0; cc < 3; ++cc) A[r][cc] += q[3] * (s->x[4 * k + r] - c[r]) * q[cc];
        }
        real *q = s->bquat + 4 * b;
        extract_rotation(A, q, K_SHAPE_ITERS);
        real R[3][3];
        quat_to_mat(q, R);
        for (uint32_t k = f; k < f + cnt; ++k) {
            const double *r = s->brest + 4 * k;
            for (int d = 0; d < 3; ++d) {
                real g = c[d] + R[d][0] * r[0] + R[d][1] * r[1] + R[d][2] * r[2];
                s->x[4 * k + d] += (g - s->x[4 * k + d]) * s->bstiff[b];
            }
        }
    }
}

/* subtract_functor (integration_kernel.cuh:465-475). */
void orc_calc_velocity(orc_system *s, double dt) {
    dt = fmin(dt, (double)s->p.max_dt);
    for (uint32_t i = 0; i < s->n; ++i) {
        for (int d = 0; d < 3; ++d) s->v[4 * i + d] = (s->x[4 * i + d] - s->x_old[4 * i + d]) / dt;
        s->v[4 * i + 3] = 0.0;
    }
}

/* XSPH (Macklin & Mueller 2013, eq. 17), normalised by the rest density:
 * v_i += c sum_j m_j (v_j - v_i) poly6(x_i - x_j) / rho0_i over the fluid
 * neighbours of the last solver iteration -- found and weighted at the
 * positions that iteration's grid was built from -- with the step's final
 * velocities (the CUDA k_xsph). */
typedef struct {
    const orc_system *s;
    uint32_t i, nb;
    uint32_t *list;
} xs_ctx;

static int xsph_visit(void *vctx, uint32_t j) {
    xs_ctx *c = (xs_ctx *)vctx;
    if (j == c->i) return 0;
    if (dist2f(c->s->sx32 + 4 * c->i, c->s->sx32 + 4 * j) < c->s->h2f &&
        c->s->sphase[j] == PBD_PHASE_FLUID) {
        if (c->nb >= c->s->p.max_neighbors) return 1;
        c->list[c->nb++] = j;
    }
    return 0;
}

void orc_apply_xsph(orc_system *s) {
    const uint32_t n = s->n;
    real *vnew = (real *)malloc(3ull * (n ? n : 1) * sizeof(real));
    const double h2 = (double)s->p.kernel_radius * (double)s->p.kernel_radius;
    set_threads();
#pragma omp parallel
    {
        uint32_t *list = (uint32_t *)malloc(s->p.max_neighbors * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1024)
        for (long long ii = 0; ii < (long long)n; ++ii) {
            uint32_t i = (uint32_t)ii, o = s->sorted_idx[i];
            for (int d = 0; d < 3; ++d) vnew[3 * i + d] = s->v[4 * o + d];
            if (s->sphase[i] != PBD_PHASE_FLUID) continue;
            xs_ctx c = {s, i, 0, list};
            int g[3];
            grid_cell(s, s->sx32 + 4 * i, g);
            for_each_candidate(s, g, s->fluid_rad, xsph_visit, &c);
            const real *xi = s->sx + 4 * i, *vi = s->v + 4 * o;
            real acc[3] = {0, 0, 0};
            for (uint32_t k = 0; k < c.nb; ++k) {
                const uint32_t j = list[k];
                const real *xj = s->sx + 4 * j, *vj = s->v + 4 * s->sorted_idx[j];
                real r2 = 0;
                for (int d = 0; d < 3; ++d) r2 += (xi[d] - xj[d]) * (xi[d] - xj[d]);
                real hm2 = h2 - r2;
                real wgt = s->poly6 * hm2 * hm2 * hm2 * (xj[3] > 0 ? 1.0 / xj[3] : (real)0.0);
                for (int d = 0; d < 3; ++d) acc[d] += (vj[d] - vi[d]) * wgt;
            }
            for (int d = 0; d < 3; ++d) vnew[3 * i + d] = vi[d] + acc[d] * ((double)s->p.xsph_c / s->srho0[i]);
        }
        free(list);
    }
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t o = s->sorted_idx[i];
        for (int d = 0; d < 3; ++d) s->v[4 * o + d] = vnew[3 * i + d];
    }
    free(vnew);
}

/* ParticleSystem::update (particlesystem.cpp:144-246), grid rebuilt at the
 * top of every iteration. */
void orc_update(orc_system *s, double dt) {
    if (!s->n) return;
    dt = fmin(dt, (double)s->p.max_dt);
    int any_fluid = 0, any_contact = 0;
    for (uint32_t i = 0; i < s->n; ++i) {
        any_fluid |= s->phase[i] == PBD_PHASE_FLUID;
        any_contact |= s->phase[i] >= PBD_PHASE_CLOTH;
    }
    int mask = DO_WORLD | ((any_fluid || s->has_gas) ? DO_FLUID : 0) | (any_contact ? DO_CONTACT : 0);
    orc_integrate(s, dt);
    for (uint32_t it = 0; it < s->p.iterations; ++it) {
        orc_build_grid(s);
        solve_pass(s, mask);
        orc_solve_distance_constraints(s);
        orc_solve_point_constraints(s);
        orc_solve_shapes(s);
    }
    orc_calc_velocity(s, dt);
    if (s->p.xsph_c != 0.f && any_fluid && s->p.iterations > 0) orc_apply_xsph(s);
}

/* ---------------------------------------------------------- accessors */

uint32_t orc_num_particles(const orc_system *s) { return s->n; }

void orc_get_positions(const orc_system *s, double *out) {
    for (size_t k = 0; k < 4ull * s->n; ++k) out[k] = R_VAL(s->x[k]);
}
void orc_get_velocities(const orc_system *s, double *out) {
    for (size_t k = 0; k < 4ull * s->n; ++k) out[k] = R_VAL(s->v[k]);
}
/* (with ORC_DUAL these set the values and clear the tangents) */
void orc_set_positions(orc_system *s, const double *p) {
    for (size_t k = 0; k < 4ull * s->n; ++k) s->x[k] = p[k];
    s->grid_valid = 0;
}
void orc_set_velocities(orc_system *s, const double *v) {
    for (size_t k = 0; k < 4ull * s->n; ++k) s->v[k] = v[k];
}

void orc_get_grid(const orc_system *s, uint32_t *sorted_hash, uint32_t *sorted_index, uint32_t *cell_start,
                  uint32_t *cell_end) {
    for (uint32_t p = 0; p < s->n; ++p) {
        if (sorted_index) sorted_index[p] = s->sorted_idx[p];
        if (sorted_hash) sorted_hash[p] = s->hash[s->sorted_idx[p]];
    }
    for (uint32_t c = 0; c < s->cells; ++c) {
        int full = s->cell_first[c + 1] > s->cell_first[c];
        if (cell_start) cell_start[c] = full ? s->cell_first[c] : 0xffffffffu;
        if (cell_end) cell_end[c] = full ? s->cell_first[c + 1] : 0u;
    }
}

void orc_get_lambdas(const orc_system *s, double *out) {
    for (uint32_t p = 0; p < s->n; ++p)
        out[s->sorted_idx[p]] = R_VAL(s->sphase[p] == PBD_PHASE_GAS ? s->glambda[p] : s->lambda[p]);
}

void orc_set_gas_open(orc_system *s, uint32_t first, uint32_t count, int open) {
    for (uint32_t k = first; k < first + count && k < s->n; ++k)
        if (s->phase[k] == PBD_PHASE_GAS) s->gas_open[k] = open ? 1 : 0;
}

void orc_set_rigid_sdf(orc_system *s, uint32_t body, const double *sdf) {
    if (body >= s->nb) return;
    for (uint32_t k = 0; k < s->bcount[body]; ++k) {
        const double *e = sdf + 4 * k;
        double *o = s->sdf + 4 * (s->bfirst[body] + k);
        if (e[3] < 0.0) {
            o[0] = o[1] = o[2] = 0.0;
            o[3] = -1.0;
            continue;
        }
        /* the CUDA path stores the FP32-normalised normal */
        const double len = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        for (int d = 0; d < 3; ++d) o[d] = (double)(float)(e[d] / len);
        o[3] = (double)(float)e[3];
    }
    s->any_sdf = 1;
}

void orc_get_forces(const orc_system *s, double *out) {
    for (size_t k = 0; k < 4ull * s->n; ++k) out[k] = R_VAL(s->force[k]);
}

void orc_set_forces(orc_system *s, const double *f) {
    for (size_t k = 0; k < 4ull * s->n; ++k) s->force[k] = f[k];
}

#ifdef ORC_DUAL
/* Seeds the direction of differentiation: tangents of the positions and
 * velocities (4n each) and of the distance-constraint stiffness (m); NULL
 * = zero. */
void orc_seed_tangents(orc_system *s, const double *dx, const double *dv, const double *dstiff) {
    for (size_t k = 0; k < 4ull * s->n; ++k) {
        s->x[k].d = dx ? dx[k] : 0.0;
        s->v[k].d = dv ? dv[k] : 0.0;
    }
    for (uint32_t c = 0; c < s->m; ++c) s->dstiff[c].d = dstiff ? dstiff[c] : 0.0;
    s->grid_valid = 0;
}

/* The directional derivatives of the positions and velocities. */
void orc_get_tangents(const orc_system *s, double *dx, double *dv) {
    for (size_t k = 0; k < 4ull * s->n; ++k) {
        if (dx) dx[k] = s->x[k].d;
        if (dv) dv[k] = s->v[k].d;
    }
}
#endif

void orc_get_neighbor_counts(const orc_system *s, uint32_t *fluid, uint32_t *contact) {
    if (fluid) memcpy(fluid, s->nb_fluid, s->n * sizeof(uint32_t));
    if (contact) memcpy(contact, s->nb_contact, s->n * sizeof(uint32_t));
}
