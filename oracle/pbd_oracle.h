/*
 * pbd_oracle.h -- CPU restatement of the reference PBD step (test
 * infrastructure only: used by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py as the checker; never by the product path).
 *
 * State and arithmetic are FP64.  The decisions the reference takes in FP32
 * -- cell hashes and every neighbour / contact distance test -- are made on
 * the FP32 rounding of the positions with the same rounding sequence as the
 * CUDA kernels, so cell lists and neighbour sets are bit-exact while the
 * projections are FP64.  Each function cites the reference lines it
 * restates.  Parameters come from pbd_params (include/pbd.h).
 */
#ifndef PBD_ORACLE_H
#define PBD_ORACLE_H

#include <stdint.h>

#include "../include/pbd.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_system orc_system;

orc_system *orc_create(const pbd_params *params, uint32_t capacity);
void orc_destroy(orc_system *s);
void orc_set_threads(int threads);
int orc_add_particles(orc_system *s, uint32_t n, const double *pos_w, const double *vel,
                      const int32_t *phase, const double *rest_density);
int orc_add_distance_constraints(orc_system *s, uint32_t m, const uint32_t *pairs,
                                 const double *rest, const double *stiffness);
int orc_add_point_constraints(orc_system *s, uint32_t p, const uint32_t *index,
                              const double *points);
int orc_add_rigid_body(orc_system *s, uint32_t first, uint32_t count, double stiffness);
void orc_set_wall_jitter(orc_system *s, const double rands[6]);

void orc_integrate(orc_system *s, double dt);
void orc_build_grid(orc_system *s);
void orc_collide(orc_system *s);
void orc_solve_fluids(orc_system *s);
void orc_collide_world(orc_system *s);
void orc_solve_distance_constraints(orc_system *s);
void orc_solve_point_constraints(orc_system *s);
void orc_solve_shapes(orc_system *s);
void orc_calc_velocity(orc_system *s, double dt);
void orc_apply_xsph(orc_system *s);
void orc_update(orc_system *s, double dt);

uint32_t orc_num_particles(const orc_system *s);
void orc_get_positions(const orc_system *s, double *out);
void orc_get_velocities(const orc_system *s, double *out);
void orc_set_positions(orc_system *s, const double *pos_w);
void orc_set_velocities(orc_system *s, const double *vel);
void orc_get_grid(const orc_system *s, uint32_t *sorted_hash, uint32_t *sorted_index,
                  uint32_t *cell_start, uint32_t *cell_end);
void orc_get_lambdas(const orc_system *s, double *out);
/* Gas phase: open / close the gas of [first, first+count); the force every
 * particle carries into the next step (4n doubles). */
void orc_set_gas_open(orc_system *s, uint32_t first, uint32_t count, int open);
void orc_get_forces(const orc_system *s, double *out);
void orc_set_forces(orc_system *s, const double *f);
/* Signed-distance data of rigid body `body` (4 doubles per particle). */
void orc_set_rigid_sdf(orc_system *s, uint32_t body, const double *sdf);
/* Neighbour count of every particle in the last fluid / contact pass. */
void orc_get_neighbor_counts(const orc_system *s, uint32_t *fluid, uint32_t *contact);
/* Only in the dual-number build (liboracle_dual.so). */
void orc_seed_tangents(orc_system *s, const double *dx, const double *dv, const double *dstiff);
void orc_get_tangents(const orc_system *s, double *dx, double *dv);

#ifdef __cplusplus
}
#endif

#endif
