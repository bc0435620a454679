// Headless driver of the reference's 2-D CPU solver (cpu/src/simulation.cpp,
// built in place from the reference tree with the stand-ins of include/):
// builds a scene of solid particles in a box and ticks it, single-threaded
// as the reference is written.  Test infrastructure: timed CPU baseline and
// invariant comparison for the 2-D granular column.
//
// The scene is assembled through Simulation's own members (access opened
// below) instead of one of its built-in init* scenes, so that the column
// of the benchmark (its lattice, jitter, friction and box) can be loaded.
// Every header outside the reference tree first, so that opening access
// below touches only the reference's own classes.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include <QHash>
#include <QList>
#include <QSet>
#include <qgl.h>
#include <GL/glu.h>
#define GLM_FORCE_RADIANS
#include <glm/vec2.hpp>
#include <glm.hpp>
#include <glm/gtx/rotate_vector.hpp>

#define private public
#include "simulation.h"
#include "gasconstraint.h"
#include "rigidcontactconstraint.h"
#include "totalfluidconstraint.h"
#include "fluidemitter.h"
#include "contactconstraint.h"
#include "boundaryconstraint.h"
#include "opensmokeemitter.h"  // last: it defines the macros H, H2, H6, H9
#undef private

#include <cstdint>

extern "C" {

void *refcpu_create(double xmin, double xmax, double ymin, double ymax, double gx, double gy) {
    Simulation *s = new Simulation();  // builds the reference's default scene
    s->clear();                        // ... which is dropped here
    s->m_counts = nullptr;
    s->m_xBoundaries = glm::dvec2(xmin, xmax);
    s->m_yBoundaries = glm::dvec2(ymin, ymax);
    s->m_gravity = glm::dvec2(gx, gy);
    return s;
}

// n solid particles: xy, v as 2n doubles (v may be NULL), unit phase SOLID.
void refcpu_add_particles(void *h, int n, const double *xy, const double *v, double mass, double s_friction,
                          double k_friction) {
    Simulation *s = static_cast<Simulation *>(h);
    for (int i = 0; i < n; ++i) {
        Particle *p = new Particle(glm::dvec2(xy[2 * i], xy[2 * i + 1]), mass, SOLID);
        if (v) p->v = glm::dvec2(v[2 * i], v[2 * i + 1]);
        p->sFriction = s_friction;
        p->kFriction = k_friction;
        s->m_particles.append(p);
    }
}

// After the last add: the tail of Simulation::init (simulation.cpp:105-108).
void refcpu_finalize(void *h) {
    Simulation *s = static_cast<Simulation *>(h);
    s->m_standardSolver.setupM(&s->m_particles);
    delete[] s->m_counts;
    s->m_counts = new int[s->m_particles.size()];
}

void refcpu_tick(void *h, double seconds, int steps) {
    Simulation *s = static_cast<Simulation *>(h);
    for (int k = 0; k < steps; ++k) s->tick(seconds);
}

int refcpu_num(void *h) { return static_cast<Simulation *>(h)->m_particles.size(); }

// xy, v: 2n doubles each (either may be NULL).
void refcpu_get(void *h, double *xy, double *v) {
    Simulation *s = static_cast<Simulation *>(h);
    for (int i = 0; i < s->m_particles.size(); ++i) {
        const Particle *p = s->m_particles.at(i);
        if (xy) {
            xy[2 * i] = p->p.x;
            xy[2 * i + 1] = p->p.y;
        }
        if (v) {
            v[2 * i] = p->v.x;
            v[2 * i + 1] = p->v.y;
        }
    }
}

void refcpu_destroy(void *h) { delete static_cast<Simulation *>(h); }

// The reference's own gas projection, GasConstraint::project
// (gasconstraint.cpp:34-134), on n 2-D particles: those with solid[i] == 0
// form one gas of rest density `density` (open or closed), the others are
// SOLID neighbours; positions are taken as the estimates, contact counts are
// zero, and project() runs `iterations` times (once per solver iteration,
// as the reference's ITERATIVE loop calls it).  xy, v: 2n doubles; imass: n
// inverse masses (0 = fixed, which the gas ignores).  Out: the estimates
// and each particle's force, 2n doubles each.  Used to pin the oracle's
// gas formulas.
void refcpu_gas_project(int n, const double *xy, const double *v, const double *imass, const int *solid,
                        double density, int open, int iterations, double *xy_out, double *f_out) {
    QList<Particle *> ps;
    QList<int> members;
    for (int i = 0; i < n; ++i) {
        Particle *p = new Particle(glm::dvec2(xy[2 * i], xy[2 * i + 1]), 1.0, solid[i] ? SOLID : GAS);
        p->imass = imass[i];
        p->ep = p->p;
        p->v = glm::dvec2(v[2 * i], v[2 * i + 1]);
        ps.append(p);
        if (!solid[i]) members.append(i);
    }
    {
        GasConstraint c(density, &members, open != 0);
        std::vector<int> counts(n, 0);
        for (int it = 0; it < iterations; ++it) c.project(&ps, counts.data());
    }
    for (int i = 0; i < n; ++i) {
        xy_out[2 * i] = ps.at(i)->ep.x;
        xy_out[2 * i + 1] = ps.at(i)->ep.y;
        f_out[2 * i] = ps.at(i)->f.x;
        f_out[2 * i + 1] = ps.at(i)->f.y;
        delete ps.at(i);
    }
}

// The reference's rigid contact, RigidContactConstraint::project
// (rigidcontactconstraint.cpp:30-96), on n 2-D SOLID particles: p are the
// start-of-step positions, ep the estimates; body[i] >= 0 puts particle i in
// that body with signed-distance data sdf[3i..3i+2] (rest-frame normal x, y,
// depth); the bodies' angles rotate the normals (Particle::getSDFData,
// particle.cpp:3-13).  Masses are height-scaled (scaleMass, particle.h:67-
// 73); each particle's count is its number of listed pairs; the pairs
// (i1 < i2) are projected once each, in order.  Out: the estimates.
void refcpu_rigid_contacts(int n, const double *p, const double *ep, const double *imass, const int *body,
                           const double *sdf, int nbodies, const double *angles, int npairs, const int *pairs,
                           double s_friction, double k_friction, double *ep_out) {
    QList<Particle *> ps;
    for (int i = 0; i < n; ++i) {
        Particle *q = new Particle(glm::dvec2(p[2 * i], p[2 * i + 1]), 1.0, SOLID);
        q->imass = imass[i];
        q->ep = glm::dvec2(ep[2 * i], ep[2 * i + 1]);
        q->bod = body[i];
        q->sFriction = s_friction;
        q->kFriction = k_friction;
        q->scaleMass();
        ps.append(q);
    }
    QList<Body *> bodies;
    for (int b = 0; b < nbodies; ++b) {
        Body *bd = new Body();
        bd->shape = nullptr;
        bd->angle = angles[b];
        bodies.append(bd);
    }
    for (int i = 0; i < n; ++i)
        if (body[i] >= 0) {
            bodies.at(body[i])->particles.append(i);
            bodies.at(body[i])->sdf[i] = SDFData(glm::dvec2(sdf[3 * i], sdf[3 * i + 1]), sdf[3 * i + 2]);
        }
    std::vector<int> counts(n, 0);
    for (int k = 0; k < npairs; ++k) {
        ++counts[pairs[2 * k]];
        ++counts[pairs[2 * k + 1]];
    }
    for (int k = 0; k < npairs; ++k) {
        RigidContactConstraint c(pairs[2 * k], pairs[2 * k + 1], &bodies, false);
        c.project(&ps, counts.data());
    }
    for (int i = 0; i < n; ++i) {
        ep_out[2 * i] = ps.at(i)->ep.x;
        ep_out[2 * i + 1] = ps.at(i)->ep.y;
        delete ps.at(i);
    }
    for (int b = 0; b < nbodies; ++b) delete bodies.at(b);
}

// The reference's fluid projection, TotalFluidConstraint::project
// (totalfluidconstraint.cpp:41-116), on n 2-D particles: those with
// fluid[i] != 0 form one fluid of rest density `density`, the others are
// SOLID; imass: n inverse masses (0 = fixed); counts: the other constraints'
// count per particle (NULL = zero).  Positions are the estimates and
// project() runs `iterations` times.  Out: the estimates (2n doubles) and
// the last call's lambda of each fluid particle (n doubles, 0 for the
// others).  Used to pin the oracle's CPU-formula flags.
void refcpu_fluid_project(int n, const double *xy, const double *imass, const int *fluid, const int *counts_in,
                          double density, int iterations, double *xy_out, double *lambda_out) {
    QList<Particle *> ps;
    QList<int> members;
    for (int i = 0; i < n; ++i) {
        Particle *p = new Particle(glm::dvec2(xy[2 * i], xy[2 * i + 1]), 1.0, fluid[i] ? FLUID : SOLID);
        p->imass = imass[i];
        p->ep = p->p;
        ps.append(p);
        if (fluid[i]) members.append(i);
    }
    {
        TotalFluidConstraint c(density, &members);
        std::vector<int> counts(n, 0);
        if (counts_in)
            for (int i = 0; i < n; ++i) counts[i] = counts_in[i];
        for (int it = 0; it < iterations; ++it) c.project(&ps, counts.data());
        for (int i = 0; i < n; ++i) lambda_out[i] = fluid[i] ? c.lambdas[i] : 0.0;
    }
    for (int i = 0; i < n; ++i) {
        xy_out[2 * i] = ps.at(i)->ep.x;
        xy_out[2 * i + 1] = ps.at(i)->ep.y;
        delete ps.at(i);
    }
}

// One FluidEmitter::tick (fluidemitter.cpp:13-77) on n 2-D particles, the
// first `members` of them FLUID members of the emitter's fluid in order
// (so that the reference's lambdas[i], read with i the member's position in
// the fluid, is the particle's own lambda), the rest SOLID.  In: positions
// p and velocities v (2n doubles), inverse masses, timers t, the members'
// lambdas, the emitter's position, rate and its two clocks (timer,
// totalTimer), the tick length and the seed of rand() (the emitter's
// frand() jitter).  Out: the particles' velocities, inverse masses, timers
// and phases (1 = FLUID, 0 = SOLID) after the tick, the clocks, and the
// emitted particles' positions and velocities (up to max_new; returns how
// many were emitted).
int refcpu_fluid_emitter_tick(int n, int members, const double *p, const double *v, const double *imass,
                              const double *t, const double *lambdas, double ex, double ey, double rate,
                              double *clocks, double secs, unsigned seed, double *v_out, double *imass_out,
                              double *t_out, int *phase_out, int max_new, double *new_p, double *new_v) {
    QList<Particle *> ps;
    QList<int> fluid;
    for (int i = 0; i < n; ++i) {
        Particle *q = new Particle(glm::dvec2(p[2 * i], p[2 * i + 1]), 1.0, i < members ? FLUID : SOLID);
        q->imass = imass[i];
        q->ep = q->p;
        q->v = glm::dvec2(v[2 * i], v[2 * i + 1]);
        q->t = t[i];
        ps.append(q);
        if (i < members) fluid.append(i);
    }
    int emitted = 0;
    {
        TotalFluidConstraint fs(1.0, &fluid);
        for (int i = 0; i < members; ++i) fs.lambdas[i] = lambdas[i];
        FluidEmitter e(glm::dvec2(ex, ey), rate, &fs);
        e.timer = clocks[0];
        e.totalTimer = clocks[1];
        srand(seed);
        e.tick(&ps, secs);
        clocks[0] = e.timer;
        clocks[1] = e.totalTimer;
        emitted = ps.size() - n;
    }
    for (int i = 0; i < ps.size(); ++i) {
        const Particle *q = ps.at(i);
        if (i < n) {
            v_out[2 * i] = q->v.x;
            v_out[2 * i + 1] = q->v.y;
            imass_out[i] = q->imass;
            t_out[i] = q->t;
            phase_out[i] = q->ph == FLUID ? 1 : 0;
        } else if (i - n < max_new) {
            new_p[2 * (i - n)] = q->p.x;
            new_p[2 * (i - n) + 1] = q->p.y;
            new_v[2 * (i - n)] = q->v.x;
            new_v[2 * (i - n) + 1] = q->v.y;
        }
        delete q;
    }
    return emitted;
}

// The reference's contact projectors on n 2-D particles (solid[i] != 0:
// SOLID, else FLUID): p the start-of-step positions, ep the estimates;
// masses height-scaled (Particle::scaleMass); the listed pairs (i1 < i2)
// become RigidContactConstraint (both SOLID, no signed-distance data) or
// ContactConstraint (simulation.cpp:186-193), the listed walls
// BoundaryConstraint (idx, isX, lower; the box's value), each particle's
// count its number of listed constraints; all projected once in order
// (pairs, then walls).  Out: the estimates.
void refcpu_contacts(int n, const double *p, const double *ep, const double *imass, const int *solid, int npairs,
                     const int *pairs, int nwalls, const int *walls, double xmin, double xmax, double ymin,
                     double ymax, double s_friction, double k_friction, double *ep_out) {
    QList<Particle *> ps;
    for (int i = 0; i < n; ++i) {
        Particle *q = new Particle(glm::dvec2(p[2 * i], p[2 * i + 1]), 1.0, solid[i] ? SOLID : FLUID);
        q->imass = imass[i];
        q->ep = glm::dvec2(ep[2 * i], ep[2 * i + 1]);
        q->sFriction = s_friction;
        q->kFriction = k_friction;
        q->scaleMass();
        ps.append(q);
    }
    QList<Body *> bodies;
    std::vector<int> counts(n, 0);
    for (int k = 0; k < npairs; ++k) {
        ++counts[pairs[2 * k]];
        ++counts[pairs[2 * k + 1]];
    }
    for (int k = 0; k < nwalls; ++k) ++counts[walls[3 * k]];
    for (int k = 0; k < npairs; ++k) {
        const int a = pairs[2 * k], b = pairs[2 * k + 1];
        if (solid[a] && solid[b]) {
            RigidContactConstraint c(a, b, &bodies, false);
            c.project(&ps, counts.data());
        } else {
            ContactConstraint c(a, b, false);
            c.project(&ps, counts.data());
        }
    }
    for (int k = 0; k < nwalls; ++k) {
        const int idx = walls[3 * k], is_x = walls[3 * k + 1], lower = walls[3 * k + 2];
        const double value = is_x ? (lower ? xmin : xmax) : (lower ? ymin : ymax);
        BoundaryConstraint c(idx, value, is_x != 0, lower != 0, false);
        c.project(&ps, counts.data());
    }
    for (int i = 0; i < n; ++i) {
        ep_out[2 * i] = ps.at(i)->ep.x;
        ep_out[2 * i + 1] = ps.at(i)->ep.y;
        delete ps.at(i);
    }
}

// The reference's own OpenSmokeEmitter::tick (opensmokeemitter.cpp:17-43)
// with its gas constraint, `ticks` ticks of `secs` after an estimates list
// of n particles: per tick the number of particles it appends to the
// estimates (counts), and for each appended particle its position, inverse
// mass, phase (1 = GAS) and whether the gas constraint took its index
// (new_* hold the first max_new).  Returns the total appended.
int refcpu_smoke_emitter_tick(int n, double ex, double ey, double rate, double secs, int ticks, int *counts,
                              int max_new, double *new_p, double *new_imass, int *new_gas, int *new_member) {
    QList<Particle *> ps;
    for (int i = 0; i < n; ++i) ps.append(new Particle(glm::dvec2(0.0, 0.0), 1.0, SOLID));
    QList<int> members;
    int total = 0;
    {
        GasConstraint gs(1.0, &members, true);
        OpenSmokeEmitter e(glm::dvec2(ex, ey), rate, &gs);
        for (int k = 0; k < ticks; ++k) {
            const int before = ps.size();
            e.tick(&ps, secs);
            counts[k] = ps.size() - before;
        }
        total = ps.size() - n;
        for (int i = n; i < ps.size(); ++i) {
            const Particle *q = ps.at(i);
            const int m = i - n;
            if (m >= max_new) break;
            new_p[2 * m] = q->p.x;
            new_p[2 * m + 1] = q->p.y;
            new_imass[m] = q->imass;
            new_gas[m] = q->ph == GAS ? 1 : 0;
            new_member[m] = gs.ps.contains(i) ? 1 : 0;
        }
        for (Particle *q : *e.getParticles()) delete q;  // the drawing-only tracers
    }
    for (Particle *q : ps) delete q;
    return total;
}

}  // extern "C"
