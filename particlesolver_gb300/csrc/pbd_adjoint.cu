// Differentiation of the PBD step: rollouts with checkpoints, and a
// backward pass of hand-written adjoint kernels for every projector of the
// step -- the integrator (predict and velocity), the PBF density / lambda
// solve and its delta with s_corr, contacts with friction, the world walls,
// distance constraints (with the gradient of every constraint's
// stiffness), pins, shape matching (through the polar rotation) and XSPH.
//
// pbd_rollout runs `steps` updates and keeps (x, v) every `every` steps in
// device memory.  pbd_backward walks the checkpoint segments from last to
// first: it restores a segment's checkpoint, recomputes the segment with
// the forward kernels while recording the positions each projector read
// (the start of every iteration, after the contact / wall pass), then runs
// the adjoint kernels in reverse.  The recomputed grids and neighbour sets
// are those of the forward pass (same kernels, same inputs), so the
// neighbour lists the forward pass used are the ones held fixed.
//
// Every adjoint is a gather: a particle sums what it receives from its own
// neighbours and constraint incidences (the contact relation and the
// constraint CSR are symmetric), so there are no atomics and results are
// deterministic.  The per-pair Jacobian blocks come from the
// scalar-generic projector formulas in pbd_dual.cuh evaluated on dual
// numbers.
#include <cmath>
#include <cstdio>

#include "pbd_dual.cuh"
#include "pbd_system.h"

namespace pbd {
namespace {

constexpr int kBlock = 256;

inline unsigned blocks_for(uint32_t n) { return (n + kBlock - 1u) / kBlock; }

__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }

// ------------------------------------------------------------ integrator

// After the last iteration: v = (x - x_old) / dt.  Given the adjoints of x
// and v after the step, the adjoint of the final positions (gfin) and the
// first part of the adjoint of x_old.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_velocity(DevParams P0, uint32_t n, float dt,
                                                         const float4 *__restrict__ gx_next,
                                                         const float4 *__restrict__ gv_next,
                                                         float4 *__restrict__ gfin, float4 *__restrict__ gxo) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float h = fminf(dt, scene_params<B>(P0, i).max_dt);
    const float4 gx = gx_next[i];
    const float4 gv = gv_next ? gv_next[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    gfin[i] = make_float4(gx.x + gv.x / h, gx.y + gv.y / h, gx.z + gv.z / h, 0.f);
    gxo[i] = make_float4(-gv.x / h, -gv.y / h, -gv.z / h, 0.f);
}

// Predict: x_old = x, x* = x + (v + g dt) dt.  gx_out = gx* + gx_old,
// gv_out = gx* dt.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_predict(DevParams P0, uint32_t n, float dt,
                                                        const float4 *__restrict__ gpred,
                                                        const float4 *__restrict__ gxo,
                                                        float4 *__restrict__ gx_out, float4 *__restrict__ gv_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float h = fminf(dt, scene_params<B>(P0, i).max_dt);
    const float4 g = gpred[i], o = gxo[i];
    gx_out[i] = make_float4(g.x + o.x, g.y + o.y, g.z + o.z, 0.f);
    gv_out[i] = make_float4(g.x * h, g.y * h, g.z * h, 0.f);
}

// ---------------------------------------------------- distance and pins

// Pins set the position: the adjoint of what the distance pass wrote is
// zero for pinned particles of active scenes.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_pins(DevParams P0, uint32_t count, uint32_t iter_left,
                                                     const uint32_t *__restrict__ particle,
                                                     const float4 *__restrict__ pin, float4 *__restrict__ gt) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const uint32_t k = particle[s];
    if (!scene_active<B>(scene_params<B>(P0, k), iter_left)) return;
    if (pin[s].w != 0.f) gt[k] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// t_k = y_k + sum_e d(y_k, y_o, s_e) / occ_k over k's incidences.  The
// adjoint of y_k gathers k's own terms and, through the same constraints
// seen from the other end, the terms of each partner o.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_distance(DevParams P0, uint32_t count, uint32_t iter_left,
                                                         const uint32_t *__restrict__ particle,
                                                         const uint32_t *__restrict__ row,
                                                         const uint32_t *__restrict__ other,
                                                         const float *__restrict__ rest,
                                                         const float *__restrict__ stiff,
                                                         const float *__restrict__ occ_of,
                                                         const float4 *__restrict__ y,
                                                         const float4 *__restrict__ gt, float4 *__restrict__ gy) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const uint32_t k = particle[s];
    const DevParams P = scene_params<B>(P0, k);
    if (!scene_active<B>(P, iter_left)) return;
    const float4 yk4 = y[k];
    const float4 gk4 = gt[k];
    const float3 gk = make_float3(gk4.x, gk4.y, gk4.z);
    const float occ_k = occ_of[k];
    float3 acc = gk;
    const uint32_t e1 = row[s + 1];
    for (uint32_t e = row[s]; e < e1; ++e) {
        const uint32_t o = other[e];
        const float4 yo4 = y[o];
        // own term: d(y_k, y_o) / occ_k, derivative in y_k
        const V3<Dual<3>> dk = distance_term<Dual<3>>(P, seed<3>(f3(yk4), 0), yk4.w, lift<Dual<3>>(f3(yo4)), yo4.w,
                                                       rest[e], cst<Dual<3>>(stiff[e]));
        acc = add3(acc, contract(dk, make_float3(gk.x / occ_k, gk.y / occ_k, gk.z / occ_k), 0));
        // partner's term: d(y_o, y_k) / occ_o, derivative in y_k
        const float4 go4 = gt[o];
        const float occ_o = occ_of[o];
        const V3<Dual<3>> dn = distance_term<Dual<3>>(P, lift<Dual<3>>(f3(yo4)), yo4.w, seed<3>(f3(yk4), 0), yk4.w,
                                                       rest[e], cst<Dual<3>>(stiff[e]));
        acc = add3(acc, contract(dn, make_float3(go4.x / occ_o, go4.y / occ_o, go4.z / occ_o), 0));
    }
    gy[k] = make_float4(acc.x, acc.y, acc.z, 0.f);
}

// d L / d stiffness_e += gt_a . d(d_a)/ds / occ_a + gt_b . d(d_b)/ds / occ_b.
// One thread per constraint accumulates over the whole backward pass.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_stiffness(DevParams P0, uint32_t m, uint32_t iter_left,
                                                          const uint32_t *__restrict__ ca,
                                                          const uint32_t *__restrict__ cb,
                                                          const float *__restrict__ crest,
                                                          const float *__restrict__ cstiff,
                                                          const float *__restrict__ occ_of,
                                                          const float4 *__restrict__ y,
                                                          const float4 *__restrict__ gt, float *__restrict__ gs) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    const uint32_t a = ca[c], b = cb[c];
    const DevParams P = scene_params<B>(P0, a);
    if (!scene_active<B>(P, iter_left)) return;
    const float4 ya = y[a], yb = y[b];
    Dual<1> st = dconst<1>(cstiff[c]);
    st.d[0] = 1.f;
    const V3<Dual<1>> da = distance_term<Dual<1>>(P, lift<Dual<1>>(f3(ya)), ya.w, lift<Dual<1>>(f3(yb)), yb.w,
                                                  crest[c], st);
    const V3<Dual<1>> db = distance_term<Dual<1>>(P, lift<Dual<1>>(f3(yb)), yb.w, lift<Dual<1>>(f3(ya)), ya.w,
                                                  crest[c], st);
    const float4 ga = gt[a], gb = gt[b];
    const float va = (ga.x * da.x.d[0] + ga.y * da.y.d[0] + ga.z * da.z.d[0]) / occ_of[a];
    const float vb = (gb.x * db.x.d[0] + gb.y * db.y.d[0] + gb.z * db.z.d[0]) / occ_of[b];
    gs[c] += va + vb;
}

// Per-constraint stiffness into the per-incidence copy the forward reads.
__global__ void __launch_bounds__(kBlock) k_scatter_stiffness(uint32_t incidences, const uint32_t *__restrict__ inc_con,
                                                              const float *__restrict__ cstiff,
                                                              float *__restrict__ stiff) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= incidences) return;
    stiff[e] = cstiff[inc_con[e]];
}

// ------------------------------------------------------ contacts + walls

__device__ __forceinline__ bool contact_test(const DevParams &P, uint32_t i, uint32_t j, int phi, int phj, float d2) {
    return j != i && d2 < P.collide2 && !(phi > kSolid && phi == phj);
}

// Walks the 27-cell contact stencil of sorted particle i (the forward
// kernel's candidate order), calling f(j) for every contact partner.
template <class F>
__device__ __forceinline__ void for_each_contact(const DevParams &P, uint32_t i, float3 pi, int phi,
                                                 const float4 *__restrict__ sx, const SortedAttr *__restrict__ sattr,
                                                 const uint32_t *__restrict__ cell_first, F &&f) {
    for_each_candidate(P, grid_pos(P, pi), 1, cell_first, [&](uint32_t j) {
        const float d2 = dist2_exact(pi, f3(sx[j]));
        if (contact_test(P, i, j, phi, sattr[j].phase, d2)) f(j);
        return true;
    });
}

// Walks the fluid neighbours of sorted particle i (|r| < h, any phase) in
// the reference's visiting order, capped at max_nb as the forward pass:
// f(j) for each.  Returns the count.
template <class F>
__device__ __forceinline__ uint32_t for_each_fluid_nb(const DevParams &P, uint32_t i, float3 pi,
                                                      const float4 *__restrict__ sx,
                                                      const uint32_t *__restrict__ cell_first, F &&f) {
    uint32_t nb = 0;
    for_each_candidate(P, grid_pos(P, pi), P.fluid_rad, cell_first, [&](uint32_t j) {
        const float d2 = dist2_exact(pi, f3(sx[j]));
        if (!(d2 < P.h2) || j == i) return true;
        if (nb >= P.max_nb) return false;
        ++nb;
        f(j);
        return true;
    });
    return nb;
}

__device__ __forceinline__ float mass_factor(const DevParams &P, float inv_wi, float wj) {
    return (P.flags & kFlagDensityNeighborMass) ? ((wj > 0.f) ? 1.f / wj : 0.f) : inv_wi;
}

// The lambda pass recomputed for sorted fluid particle i, keeping its sums
// for the adjoint: fl1 = (sum of neighbour density terms, sum |sg|^2,
// lambda, neighbour count), fl2 = (grad = -sum sg, divisor of the delta
// pass).  Other particles: lambda 0.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_fluid_lambda(DevParams P0, uint32_t n, const float4 *__restrict__ sx,
                                                             const SortedAttr *__restrict__ sattr,
                                                             const uint32_t *__restrict__ cell_first,
                                                             float4 *__restrict__ fl1, float4 *__restrict__ fl2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    const SortedAttr a = sattr[i];
    if (a.phase != kFluid) {
        fl1[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        fl2[i] = make_float4(0.f, 0.f, 0.f, 1.f);
        return;
    }
    const float4 pi4 = sx[i];
    const float3 pi = f3(pi4);
    const float inv_w = 1.f / pi4.w, inv_rho0 = 1.f / a.rho0;
    const float spiky_r = -P.spiky * inv_rho0;
    float ro = 0.f, denom = 0.f;
    V3<float> grad{0.f, 0.f, 0.f};
    const uint32_t nb = for_each_fluid_nb(P, i, pi, sx, cell_first, [&](uint32_t j) {
        const float4 pj4 = sx[j];
        const LambdaTerm<float> t = lambda_term<float>(P, lift<float>(pi), lift<float>(f3(pj4)),
                                                       mass_factor(P, inv_w, pj4.w), spiky_r);
        const float sw = density_weight(P, sattr, j);
        ro += t.ro * sw;
        denom += gdot(t.sg, t.sg);
        grad = grad - t.sg * sw;
    });
    const float lam = lambda_of<float>(P, ro, denom, grad, inv_w, inv_rho0);
    const float div = (P.flags & kFlagDeltaOverRho0) ? a.rho0 : a.rho0 + (float)nb;
    fl1[i] = make_float4(ro, denom, lam, (float)nb);
    fl2[i] = make_float4(grad.x, grad.y, grad.z, div);
}

// Forward of the fused pass for sorted particle i: u = x_i + its fluid
// delta (fluid) or its contact terms (phases >= CLOTH), then walls.  The
// adjoint of u from the adjoint gy of the written position, and the walls'
// part of the adjoint of x_old; stores u's adjoint and i's contact count.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_solve_prep(DevParams P0, uint32_t n, uint32_t iter_left,
                                                           bool contacts, bool fluids, const float4 *__restrict__ sx,
                                                           const SortedAttr *__restrict__ sattr,
                                                           const uint32_t *__restrict__ sidx,
                                                           const uint32_t *__restrict__ cell_first,
                                                           const float4 *__restrict__ x_old,
                                                           const float4 *__restrict__ fl1,
                                                           const float4 *__restrict__ fl2,
                                                           const float4 *__restrict__ gy,
                                                           float4 *__restrict__ gu, uint32_t *__restrict__ cnt,
                                                           float4 *__restrict__ gxo) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    const uint32_t orig = sidx[i];
    const float4 g4 = gy[orig];
    if (!scene_active<B>(P, iter_left)) {
        gu[i] = g4;
        cnt[i] = 0u;
        return;
    }
    const float4 pi4 = sx[i];
    const float3 pi = f3(pi4);
    const int phi = sattr[i].phase;
    const float3 prev = f3(x_old[orig]);
    float3 u = pi;
    uint32_t nb = 0;
    if (fluids && phi == kFluid) {
        const float lam_i = fl1[i].z, div = fl2[i].w;
        const float poly6_ref = P.poly6 * P.scorr_inv_ref;
        V3<float> acc{0.f, 0.f, 0.f};
        for_each_fluid_nb(P, i, pi, sx, cell_first, [&](uint32_t j) {
            acc = acc + delta_term<float>(P, lift<float>(pi), lift<float>(f3(sx[j])), lam_i + fl1[j].z, poly6_ref);
        });
        u = make_float3(pi.x + acc.x / div, pi.y + acc.y / div, pi.z + acc.z / div);
    } else if (contacts && phi >= kCloth) {
        for_each_contact(P, i, pi, phi, sx, sattr, cell_first, [&](uint32_t) { ++nb; });
        if (nb) {
            V3<float> acc = lift<float>(make_float3(0.f, 0.f, 0.f));
            const float fnb = (float)nb;
            for_each_contact(P, i, pi, phi, sx, sattr, cell_first, [&](uint32_t j) {
                const float4 pj4 = sx[j];
                acc = acc + contact_pair<float>(P, lift<float>(pi), pi4.w, phi, lift<float>(prev), lift<float>(f3(pj4)),
                                                pj4.w, sattr[j].phase, lift<float>(f3(x_old[sidx[j]])), fnb);
            });
            u = make_float3(pi.x + acc.x, pi.y + acc.y, pi.z + acc.z);
        }
    }
    cnt[i] = nb;
    const V3<Dual<6>> w = world_generic<Dual<6>>(P, seed<6>(u, 0), phi, seed<6>(prev, 3));
    const float3 g = make_float3(g4.x, g4.y, g4.z);
    const float3 gu3 = contract(w, g, 0);
    const float3 go3 = contract(w, g, 3);
    gu[i] = make_float4(gu3.x, gu3.y, gu3.z, 0.f);
    const float4 o = gxo[orig];
    gxo[orig] = make_float4(o.x + go3.x, o.y + go3.y, o.z + go3.z, 0.f);
}

// d delta_term / d lambda_sum: the direction a unit of lambda moves i.
__device__ __forceinline__ float3 delta_dlam(const DevParams &P, float3 pi, float3 pj, float lam_sum, float poly6_ref) {
    Dual<1> l = dconst<1>(lam_sum);
    l.d[0] = 1.f;
    const V3<Dual<1>> t = delta_term<Dual<1>>(P, lift<Dual<1>>(pi), lift<Dual<1>>(pj), l, poly6_ref);
    return make_float3(t.x.d[0], t.y.d[0], t.z.d[0]);
}

// Adjoint of lambda_i: lambda_i enters i's own delta and the delta of
// every fluid neighbour j (lambda_i + lambda_j).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_fluid_lbar(DevParams P0, uint32_t n, uint32_t iter_left,
                                                           const float4 *__restrict__ sx,
                                                           const SortedAttr *__restrict__ sattr,
                                                           const uint32_t *__restrict__ cell_first,
                                                           const float4 *__restrict__ fl1,
                                                           const float4 *__restrict__ fl2,
                                                           const float4 *__restrict__ gu, float *__restrict__ lbar) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    if (!scene_active<B>(P, iter_left) || sattr[i].phase != kFluid) {
        lbar[i] = 0.f;
        return;
    }
    const float3 pi = f3(sx[i]);
    const float lam_i = fl1[i].z, div_i = fl2[i].w;
    const float4 gi4 = gu[i];
    const float poly6_ref = P.poly6 * P.scorr_inv_ref;
    float acc = 0.f;
    for_each_fluid_nb(P, i, pi, sx, cell_first, [&](uint32_t j) {
        const float3 pj = f3(sx[j]);
        const float lam_j = fl1[j].z;
        const float3 a = delta_dlam(P, pi, pj, lam_i + lam_j, poly6_ref);
        acc += (gi4.x * a.x + gi4.y * a.y + gi4.z * a.z) / div_i;
        if (sattr[j].phase == kFluid) {
            const float3 b = delta_dlam(P, pj, pi, lam_j + lam_i, poly6_ref);
            const float4 gj4 = gu[j];
            acc += (gj4.x * b.x + gj4.y * b.y + gj4.z * b.z) / fl2[j].w;
        }
    });
    lbar[i] = acc;
}

// Gather for sorted particle j: the adjoint of its start-of-iteration
// position -- identity, plus its own contact / fluid delta terms and its
// own lambda, plus every partner's contact term, fluid delta term and
// lambda through x_j -- and the contact terms' part of the adjoint of
// x_old_j.  A partner's lambda in x_j comes from perturbing only the pair
// (i, j) term of its kept sums.  CONTACTS / FLUIDS: the scene has contact
// particles / fluid (compile-time, so each variant carries only the dual
// code it needs).
template <bool B, bool CONTACTS, bool FLUIDS>
__global__ void __launch_bounds__(kBlock) k_adj_solve_gather(DevParams P0, uint32_t n, uint32_t iter_left,
                                                             const float4 *__restrict__ sx,
                                                             const SortedAttr *__restrict__ sattr,
                                                             const uint32_t *__restrict__ sidx,
                                                             const uint32_t *__restrict__ cell_first,
                                                             const float4 *__restrict__ x_old,
                                                             const float4 *__restrict__ fl1,
                                                             const float4 *__restrict__ fl2,
                                                             const float *__restrict__ lbar,
                                                             const float4 *__restrict__ gu,
                                                             const uint32_t *__restrict__ cnt,
                                                             float4 *__restrict__ gstart, float4 *__restrict__ gxo) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const DevParams P = scene_params<B>(P0, j);
    const uint32_t orig = sidx[j];
    const float4 guj4 = gu[j];
    const float3 guj = make_float3(guj4.x, guj4.y, guj4.z);
    if (!scene_active<B>(P, iter_left) || !(CONTACTS || FLUIDS)) {
        gstart[orig] = make_float4(guj.x, guj.y, guj.z, 0.f);
        return;
    }
    const float4 pj4 = sx[j];
    const float3 pj = f3(pj4);
    const int phj = sattr[j].phase;
    const float3 prevj = f3(x_old[orig]);
    float3 gx = guj, go = make_float3(0.f, 0.f, 0.f);
    if (CONTACTS) {
        const uint32_t nj = cnt[j];
        for_each_contact(P, j, pj, phj, sx, sattr, cell_first, [&](uint32_t i) {
            const float4 pi4 = sx[i];
            const int phi = sattr[i].phase;
            const float3 previ = f3(x_old[sidx[i]]);
            if (phj >= kCloth && phj != kFluid && nj) {  // j's own term c_ji, in x_j and x_old_j
                const V3<Dual<6>> c = contact_pair<Dual<6>>(P, seed<6>(pj, 0), pj4.w, phj, seed<6>(prevj, 3),
                                                            lift<Dual<6>>(f3(pi4)), pi4.w, phi, lift<Dual<6>>(previ),
                                                            (float)nj);
                gx = add3(gx, contract(c, guj, 0));
                go = add3(go, contract(c, guj, 3));
            }
            const uint32_t ni = cnt[i];
            if (phi >= kCloth && ni) {  // partner's term c_ij, in x_j and x_old_j
                const float4 gui4 = gu[i];
                const float3 gui = make_float3(gui4.x, gui4.y, gui4.z);
                const V3<Dual<6>> c = contact_pair<Dual<6>>(P, lift<Dual<6>>(f3(pi4)), pi4.w, phi,
                                                            lift<Dual<6>>(previ), seed<6>(pj, 0), pj4.w, phj,
                                                            seed<6>(prevj, 3), (float)ni);
                gx = add3(gx, contract(c, gui, 0));
                go = add3(go, contract(c, gui, 3));
            }
        });
    }
    if (FLUIDS) {
        const float poly6_ref = P.poly6 * P.scorr_inv_ref;
        const bool jf = phj == kFluid;
        const float lam_j = fl1[j].z, div_j = fl2[j].w, lbar_j = lbar[j];
        const float inv_wj = 1.f / pj4.w;
        const float inv_rho0_j = 1.f / sattr[j].rho0;
        // own lambda_j in x_j: the whole sum on dual numbers
        Dual<3> ro = dconst<3>(0.f), denom = dconst<3>(0.f);
        V3<Dual<3>> grad = lift<Dual<3>>(make_float3(0.f, 0.f, 0.f));
        const V3<Dual<3>> pjd = seed<3>(pj, 0);
        for_each_fluid_nb(P, j, pj, sx, cell_first, [&](uint32_t i) {
            const float4 pi4 = sx[i];
            const float3 pi = f3(pi4);
            const float lam_i = fl1[i].z;
            if (jf) {
                // own delta term, in x_j
                const V3<Dual<3>> t = delta_term<Dual<3>>(P, pjd, lift<Dual<3>>(pi), cst<Dual<3>>(lam_j + lam_i),
                                                          poly6_ref);
                gx = add3(gx, contract(t, make_float3(guj.x / div_j, guj.y / div_j, guj.z / div_j), 0));
                const LambdaTerm<Dual<3>> lt =
                    lambda_term<Dual<3>>(P, pjd, lift<Dual<3>>(pi), mass_factor(P, inv_wj, pi4.w), -P.spiky * inv_rho0_j);
                const float sw = density_weight(P, sattr, i);
                ro = ro + lt.ro * sw;
                denom = denom + gdot(lt.sg, lt.sg);
                grad = grad - lt.sg * sw;
            }
            if (sattr[i].phase == kFluid) {
                // partner's delta term, in x_j
                const float div_i = fl2[i].w;
                const float4 gui4 = gu[i];
                const V3<Dual<3>> t = delta_term<Dual<3>>(P, lift<Dual<3>>(pi), pjd, cst<Dual<3>>(lam_i + lam_j),
                                                          poly6_ref);
                gx = add3(gx, contract(t, make_float3(gui4.x / div_i, gui4.y / div_i, gui4.z / div_i), 0));
                // partner's lambda, in x_j: only the (i, j) term of its sums moves
                const float inv_wi = 1.f / pi4.w, inv_rho0_i = 1.f / sattr[i].rho0;
                const float mf = mass_factor(P, inv_wi, pj4.w), sr = -P.spiky * inv_rho0_i;
                const LambdaTerm<float> tv = lambda_term<float>(P, lift<float>(pi), lift<float>(pj), mf, sr);
                const LambdaTerm<Dual<3>> td = lambda_term<Dual<3>>(P, lift<Dual<3>>(pi), pjd, mf, sr);
                const float sw = density_weight(P, sattr, j);  // j's weight in i's sums
                const float4 s1 = fl1[i], s2 = fl2[i];
                const Dual<3> ro_i = cst<Dual<3>>(s1.x - tv.ro * sw) + td.ro * sw;
                const Dual<3> de_i = cst<Dual<3>>(s1.y - gdot(tv.sg, tv.sg)) + gdot(td.sg, td.sg);
                const V3<Dual<3>> gr_i =
                    lift<Dual<3>>(make_float3(s2.x + sw * tv.sg.x, s2.y + sw * tv.sg.y, s2.z + sw * tv.sg.z)) - td.sg * sw;
                const Dual<3> li = lambda_of<Dual<3>>(P, ro_i, de_i, gr_i, inv_wi, inv_rho0_i);
                const float lb = lbar[i];
                gx = make_float3(gx.x + lb * li.d[0], gx.y + lb * li.d[1], gx.z + lb * li.d[2]);
            }
        });
        if (jf) {
            const Dual<3> lj = lambda_of<Dual<3>>(P, ro, denom, grad, inv_wj, inv_rho0_j);
            gx = make_float3(gx.x + lbar_j * lj.d[0], gx.y + lbar_j * lj.d[1], gx.z + lbar_j * lj.d[2]);
        }
    }
    gstart[orig] = make_float4(gx.x, gx.y, gx.z, 0.f);
    if (CONTACTS) {
        const float4 o = gxo[orig];
        gxo[orig] = make_float4(o.x + go.x, o.y + go.y, o.z + go.z, 0.f);
    }
}

// ---------------------------------------------------------- shape matching

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Polar rotation of A (the forward kernel's extraction, Mueller, Bender,
// Chentanez, Macklin 2016), run from the identity to convergence.
__device__ void polar_rotation(const float A[3][3], float R[3][3]) {
    float q[4] = {0.f, 0.f, 0.f, 1.f};
    for (int it = 0; it < 64; ++it) {
        float M[3][3];
        const float xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
        const float xy = q[0] * q[1], xz = q[0] * q[2], yz = q[1] * q[2];
        const float wx = q[3] * q[0], wy = q[3] * q[1], wz = q[3] * q[2];
        M[0][0] = 1.f - 2.f * (yy + zz); M[0][1] = 2.f * (xy - wz);       M[0][2] = 2.f * (xz + wy);
        M[1][0] = 2.f * (xy + wz);       M[1][1] = 1.f - 2.f * (xx + zz); M[1][2] = 2.f * (yz - wx);
        M[2][0] = 2.f * (xz - wy);       M[2][1] = 2.f * (yz + wx);       M[2][2] = 1.f - 2.f * (xx + yy);
        float ox = 0.f, oy = 0.f, oz = 0.f, dsum = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float rx = M[0][c], ry = M[1][c], rz = M[2][c];
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
        const float wl = sqrtf(ox * ox + oy * oy + oz * oz);
        if (wl < 1.0e-9f) break;
        const float sh = sinf(0.5f * wl) / wl, ch = cosf(0.5f * wl);
        const float d[4] = {ox * sh, oy * sh, oz * sh, ch};
        float r[4];
        r[3] = d[3] * q[3] - d[0] * q[0] - d[1] * q[1] - d[2] * q[2];
        r[0] = d[3] * q[0] + d[0] * q[3] + d[1] * q[2] - d[2] * q[1];
        r[1] = d[3] * q[1] - d[0] * q[2] + d[1] * q[3] + d[2] * q[0];
        r[2] = d[3] * q[2] + d[0] * q[1] - d[1] * q[0] + d[2] * q[3];
        const float qn = rsqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
        for (int k = 0; k < 4; ++k) q[k] = r[k] * qn;
    }
    const float xx = q[0] * q[0], yy = q[1] * q[1], zz = q[2] * q[2];
    const float xy = q[0] * q[1], xz = q[0] * q[2], yz = q[1] * q[2];
    const float wx = q[3] * q[0], wy = q[3] * q[1], wz = q[3] * q[2];
    R[0][0] = 1.f - 2.f * (yy + zz); R[0][1] = 2.f * (xy - wz);       R[0][2] = 2.f * (xz + wy);
    R[1][0] = 2.f * (xy + wz);       R[1][1] = 1.f - 2.f * (xx + zz); R[1][2] = 2.f * (yz - wx);
    R[2][0] = 2.f * (xz - wy);       R[2][1] = 2.f * (yz + wx);       R[2][2] = 1.f - 2.f * (xx + yy);
}

// Shape matching (k_shapes): x'_k = x_k + s (c + R q_k - x_k), c the
// mass-weighted centre, R the polar rotation of A = sum m_k (x_k - c) q_k^T.
// Adjoint, one warp per body, g the adjoint of x' (in place):
//   cbar = s sum g_k,  Rbar = s sum g_k q_k^T,
//   Abar = R [y]x with (tr S I - S) y = vee(R^T Rbar - Rbar^T R), S = R^T A
//   (the derivative of the polar rotation),
//   xbar_k = (1 - s) g_k + m_k / M cbar + m_k Abar q_k
// (the centre's part of A vanishes: sum m_k q_k = 0 by construction).
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_shapes(DevParams P0, uint32_t iter_left, uint32_t bodies,
                                                       const uint4 *__restrict__ range, const float *__restrict__ stiff,
                                                       const float4 *__restrict__ rest, const float4 *__restrict__ x,
                                                       float4 *__restrict__ g) {
    const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= bodies) return;
    const uint4 rg = range[b];
    const uint32_t first = rg.x, count = rg.y, roff = rg.z;
    if (!scene_active<B>(scene_params<B>(P0, first), iter_left)) return;
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
    sx = wsum(sx);
    sy = wsum(sy);
    sz = wsum(sz);
    sm = wsum(sm);
    const float3 c = make_float3(o.x + sx / sm, o.y + sy / sm, o.z + sz / sm);
    float A[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float Rb[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float cb[3] = {0.f, 0.f, 0.f};
    for (uint32_t k = lane; k < count; k += 32) {
        const float4 p = x[first + k];
        const float4 q = rest[roff + k];
        const float4 gk = g[first + k];
        const float d[3] = {q.w * (p.x - c.x), q.w * (p.y - c.y), q.w * (p.z - c.z)};
        const float gg[3] = {gk.x, gk.y, gk.z};
        const float qq[3] = {q.x, q.y, q.z};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            cb[r] += gg[r];
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                A[r][cc] += d[r] * qq[cc];
                Rb[r][cc] += gg[r] * qq[cc];
            }
        }
    }
    const float st = stiff[b];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        cb[r] = wsum(cb[r]) * st;
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            A[r][cc] = wsum(A[r][cc]);
            Rb[r][cc] = wsum(Rb[r][cc]) * st;
        }
    }
    float R[3][3];
    polar_rotation(A, R);
    // S = sym(R^T A), M = R^T Rbar
    float S[3][3], M[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            float sa = 0.f, mm = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                sa += R[k][r] * A[k][cc];
                mm += R[k][r] * Rb[k][cc];
            }
            S[r][cc] = sa;
            M[r][cc] = mm;
        }
    const float u[3] = {M[2][1] - M[1][2], M[0][2] - M[2][0], M[1][0] - M[0][1]};
    const float tr = S[0][0] + S[1][1] + S[2][2];
    float K[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) K[r][cc] = ((r == cc) ? tr : 0.f) - 0.5f * (S[r][cc] + S[cc][r]);
    // y = K^-1 u by the adjugate (K symmetric positive definite for a
    // non-degenerate body)
    const float c00 = K[1][1] * K[2][2] - K[1][2] * K[2][1], c01 = K[1][2] * K[2][0] - K[1][0] * K[2][2],
                c02 = K[1][0] * K[2][1] - K[1][1] * K[2][0];
    const float det = K[0][0] * c00 + K[0][1] * c01 + K[0][2] * c02;
    const float id = (fabsf(det) > 1e-20f) ? 1.f / det : 0.f;
    const float Ki[3][3] = {
        {c00 * id, (K[0][2] * K[2][1] - K[0][1] * K[2][2]) * id, (K[0][1] * K[1][2] - K[0][2] * K[1][1]) * id},
        {c01 * id, (K[0][0] * K[2][2] - K[0][2] * K[2][0]) * id, (K[0][2] * K[1][0] - K[0][0] * K[1][2]) * id},
        {c02 * id, (K[0][1] * K[2][0] - K[0][0] * K[2][1]) * id, (K[0][0] * K[1][1] - K[0][1] * K[1][0]) * id}};
    const float y[3] = {Ki[0][0] * u[0] + Ki[0][1] * u[1] + Ki[0][2] * u[2],
                        Ki[1][0] * u[0] + Ki[1][1] * u[1] + Ki[1][2] * u[2],
                        Ki[2][0] * u[0] + Ki[2][1] * u[1] + Ki[2][2] * u[2]};
    const float Y[3][3] = {{0.f, -y[2], y[1]}, {y[2], 0.f, -y[0]}, {-y[1], y[0], 0.f}};
    float Ab[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) Ab[r][cc] = R[r][0] * Y[0][cc] + R[r][1] * Y[1][cc] + R[r][2] * Y[2][cc];
    for (uint32_t k = lane; k < count; k += 32) {
        const float4 q = rest[roff + k];
        const float4 gk = g[first + k];
        const float m = q.w, mf = q.w / sm;
        const float ax = Ab[0][0] * q.x + Ab[0][1] * q.y + Ab[0][2] * q.z;
        const float ay = Ab[1][0] * q.x + Ab[1][1] * q.y + Ab[1][2] * q.z;
        const float az = Ab[2][0] * q.x + Ab[2][1] * q.y + Ab[2][2] * q.z;
        g[first + k] = make_float4((1.f - st) * gk.x + mf * cb[0] + m * ax, (1.f - st) * gk.y + mf * cb[1] + m * ay,
                                   (1.f - st) * gk.z + mf * cb[2] + m * az, 0.f);
    }
}

// ------------------------------------------------------------------ XSPH

// XSPH (k_xsph) over the last iteration's grid: for fluid i,
// v'_i = v_i + (c / rho0_i) sum_j m_j (v_j - v_i) W(x_i - x_j) over fluid
// neighbours.  Given the adjoint g of v' (sorted, gvs), the adjoint of v
// (written to gv_out, original order) and of the positions (added to gx_out,
// original order).  vs: velocities before XSPH, sorted.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_xsph(DevParams P0, uint32_t n, const float4 *__restrict__ sx,
                                                     const SortedAttr *__restrict__ sattr,
                                                     const uint32_t *__restrict__ sidx,
                                                     const uint32_t *__restrict__ cell_first,
                                                     const float4 *__restrict__ vs, const float4 *__restrict__ gvs,
                                                     float4 *__restrict__ gv_out, float4 *__restrict__ gx_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevParams P = scene_params<B>(P0, i);
    const uint32_t orig = sidx[i];
    const float4 gi4 = gvs[i];
    const bool fi = sattr[i].phase == kFluid && P.xsph_c != 0.f && P.iterations > 0u;
    if (!fi) {
        gv_out[orig] = gi4;
        gx_out[orig] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 xi4 = sx[i];
    const float3 xi = f3(xi4);
    const float3 vi = f3(vs[i]);
    const float3 gi = f3(gi4);
    const float ci = P.xsph_c / sattr[i].rho0;
    const float mi = (xi4.w > 0.f) ? 1.f / xi4.w : 0.f;
    float3 gv = gi, gx = make_float3(0.f, 0.f, 0.f);
    const V3<Dual<3>> xid = seed<3>(xi, 0);
    uint32_t nb = 0;
    for_each_candidate(P, grid_pos(P, xi), P.fluid_rad, cell_first, [&](uint32_t j) {
        const float4 xj4 = sx[j];
        const float d2 = dist2_exact(xi, f3(xj4));
        if (!(d2 < P.h2) || j == i || sattr[j].phase != kFluid) return true;
        if (nb >= P.max_nb) return false;
        ++nb;
        const float3 vj = f3(vs[j]);
        const float3 gj = f3(gvs[j]);
        const float cj = P.xsph_c / sattr[j].rho0;
        const float mj = (xj4.w > 0.f) ? 1.f / xj4.w : 0.f;
        const V3<Dual<3>> dr = xid - lift<Dual<3>>(f3(xj4));
        const Dual<3> hm2 = P.h2 - gdot(dr, dr);
        const Dual<3> W = hm2 * hm2 * hm2 * P.poly6;
        // own: v'_i += ci mj (vj - vi) W
        gv = make_float3(gv.x - gi.x * ci * mj * W.v, gv.y - gi.y * ci * mj * W.v, gv.z - gi.z * ci * mj * W.v);
        const float own = ci * mj * (gi.x * (vj.x - vi.x) + gi.y * (vj.y - vi.y) + gi.z * (vj.z - vi.z));
        // partner: v'_j += cj mi (vi - vj) W (the same W, symmetric in x)
        gv = make_float3(gv.x + gj.x * cj * mi * W.v, gv.y + gj.y * cj * mi * W.v, gv.z + gj.z * cj * mi * W.v);
        const float par = cj * mi * (gj.x * (vi.x - vj.x) + gj.y * (vi.y - vj.y) + gj.z * (vi.z - vj.z));
        const float k = own + par;
        gx = make_float3(gx.x + k * W.d[0], gx.y + k * W.d[1], gx.z + k * W.d[2]);
        return true;
    });
    gv_out[orig] = make_float4(gv.x, gv.y, gv.z, 0.f);
    gx_out[orig] = make_float4(gx.x, gx.y, gx.z, 0.f);
}

// Sorted copies for the XSPH adjoint: vs = v_before[sidx], gvs = g[sidx].
__global__ void __launch_bounds__(kBlock) k_adj_gather_sorted(uint32_t n, const uint32_t *__restrict__ sidx,
                                                              const float4 *__restrict__ a, const float4 *__restrict__ b,
                                                              float4 *__restrict__ as, float4 *__restrict__ bs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = sidx[i];
    as[i] = a[o];
    bs[i] = b[o];
}

// v before XSPH: (x_fin - x_old) / min(dt, max_dt), as k_velocity.
template <bool B>
__global__ void __launch_bounds__(kBlock) k_adj_vel_of(DevParams P0, uint32_t n, float dt,
                                                       const float4 *__restrict__ xfin,
                                                       const float4 *__restrict__ xold, float4 *__restrict__ v) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = xfin[i], o = xold[i];
    const float nd = -fminf(dt, scene_params<B>(P0, i).max_dt);
    v[i] = make_float4((o.x - p.x) / nd, (o.y - p.y) / nd, (o.z - p.z) / nd, 0.f);
}

__global__ void __launch_bounds__(kBlock) k_add4(uint32_t n, float4 *__restrict__ a, const float4 *__restrict__ b) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = a[i], y = b[i];
    a[i] = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, 0.f);
}

// ------------------------------------------------------------ host side

#define ADJ_TRY(s, call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return pbd_internal_fail((s), PBD_ERR_CUDA, std::string(#call " failed: ") + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
cudaError_t grow(T **p, size_t &have, size_t want) {
    if (have >= want && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    have = 0;
    cudaError_t e = cudaMalloc((void **)p, want * sizeof(T));
    if (e == cudaSuccess) have = want;
    return e;
}

// The adjoint covers every stage of the step except the gas phase, the
// signed-distance rigid contact and the CPU reference's PBF and contact
// rules.
int differentiable(pbd_system *s) {
    if (s->n_gas)
        return pbd_internal_fail(s, PBD_ERR_UNSUPPORTED, "the adjoint does not cover the gas phase (the system holds gas particles)");
    if (s->any_sdf)
        return pbd_internal_fail(s, PBD_ERR_UNSUPPORTED, "the adjoint does not cover the signed-distance rigid contact (a body has sdf data)");
    for (const pbd_scene &sc : s->scenes)
        if (sc.params.flags & (PBD_FLAG_SKIP_FIXED_NEIGHBORS | PBD_FLAG_DELTA_OVER_COUNT | PBD_FLAG_CPU_CONTACTS))
            return pbd_internal_fail(s, PBD_ERR_UNSUPPORTED,
                                     "the adjoint does not cover the CPU reference's PBF neighbour and divisor rules "
                                     "or its contact projectors (PBD_FLAG_SKIP_FIXED_NEIGHBORS, "
                                     "PBD_FLAG_DELTA_OVER_COUNT, PBD_FLAG_CPU_CONTACTS)");
    return PBD_OK;
}

}  // namespace
}  // namespace pbd

using namespace pbd;

void pbd_internal_free_adjoint(pbd_system *s) {
    auto &a = s->adj;
    for (float4 **p : {&a.ckpt_x, &a.ckpt_v, &a.ckpt_q, &a.rec, &a.gx, &a.gv, &a.gxo, &a.gt, &a.gy, &a.gu,
                       &a.save_x, &a.save_v, &a.save_xo, &a.fl1, &a.fl2, &a.w1, &a.w2, &a.w3}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    if (a.cnt) cudaFree(a.cnt);
    if (a.gstiff) cudaFree(a.gstiff);
    if (a.lbar) cudaFree(a.lbar);
    a.cnt = nullptr;
    a.gstiff = nullptr;
    a.lbar = nullptr;
    a.ckpt_cap = a.rec_cap = a.ckpt_q_cap = 0;
    a.work_cap = a.stiff_cap = 0;
    a.recorded = false;
}

extern "C" {

int pbd_set_distance_stiffness(pbd_system *s, uint32_t count, const float *stiffness, int on_device, void *stream) {
    if (int rc = pbd_internal_guard(s)) return rc;
    const uint32_t m = (uint32_t)s->dist_a.size();
    if (count != m) return pbd_internal_fail(s, PBD_ERR_INVALID_ARGUMENT, "stiffness count must equal the number of distance constraints");
    if (m == 0) return PBD_OK;
    if (!stiffness) return pbd_internal_fail(s, PBD_ERR_INVALID_ARGUMENT, "stiffness is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> host(m);
    if (on_device) {
        ADJ_TRY(s, cudaMemcpyAsync(host.data(), stiffness, m * 4ull, cudaMemcpyDeviceToHost, st));
        ADJ_TRY(s, cudaStreamSynchronize(st));
    } else {
        std::copy(stiffness, stiffness + m, host.begin());
    }
    for (uint32_t c = 0; c < m; ++c)
        if (!(host[c] >= 0.f && host[c] <= 1.f))
            return pbd_internal_fail(s, PBD_ERR_INVALID_ARGUMENT, "stiffness must be in [0, 1]");
    s->dist_stiff = host;
    ++s->version;
    const ConstraintBuffers &c = s->cons;
    ADJ_TRY(s, cudaMemcpyAsync(c.con_stiff, host.data(), m * 4ull, cudaMemcpyHostToDevice, st));
    uint32_t E = 0;
    ADJ_TRY(s, cudaMemcpyAsync(&E, c.row + c.count, 4, cudaMemcpyDeviceToHost, st));
    ADJ_TRY(s, cudaStreamSynchronize(st));
    if (E) k_scatter_stiffness<<<blocks_for(E), kBlock, 0, st>>>(E, c.inc_con, c.con_stiff, c.stiff);
    ADJ_TRY(s, cudaGetLastError());
    ADJ_TRY(s, cudaStreamSynchronize(st));
    return PBD_OK;
}

uint32_t pbd_num_distance_constraints(const pbd_system *s) { return s ? (uint32_t)s->dist_a.size() : 0u; }

int pbd_rollout(pbd_system *s, float dt, uint32_t steps, uint32_t every, void *stream) {
    if (int rc = pbd_internal_guard(s)) return rc;
    if (!(dt > 0.f) || !std::isfinite(dt)) return pbd_internal_fail(s, PBD_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (steps == 0 || every == 0) return pbd_internal_fail(s, PBD_ERR_INVALID_ARGUMENT, "steps and every must be > 0");
    if (int rc = differentiable(s)) return rc;
    auto &a = s->adj;
    a.recorded = false;
    const uint32_t n = s->n;
    const uint32_t nck = (steps + every - 1u) / every;
    const size_t want = (size_t)nck * n;
    if (a.ckpt_cap < want || !a.ckpt_x || !a.ckpt_v) {
        if (a.ckpt_x) cudaFree(a.ckpt_x);
        if (a.ckpt_v) cudaFree(a.ckpt_v);
        a.ckpt_x = a.ckpt_v = nullptr;
        a.ckpt_cap = 0;
        ADJ_TRY(s, cudaMalloc((void **)&a.ckpt_x, want * sizeof(float4)));
        ADJ_TRY(s, cudaMalloc((void **)&a.ckpt_v, want * sizeof(float4)));
        a.ckpt_cap = want;
    }
    const uint32_t nb = s->bodies.count;
    const size_t want_q = (size_t)nck * nb + nb;  // checkpoints + the final rotations
    if (nb && (a.ckpt_q_cap < want_q || !a.ckpt_q)) {
        if (a.ckpt_q) cudaFree(a.ckpt_q);
        a.ckpt_q = nullptr;
        a.ckpt_q_cap = 0;
        ADJ_TRY(s, cudaMalloc((void **)&a.ckpt_q, want_q * sizeof(float4)));
        a.ckpt_q_cap = want_q;
    }
    cudaStream_t st = (cudaStream_t)stream;
    dt = pbd_internal_clamp_dt(s, dt);
    const size_t bytes = (size_t)n * sizeof(float4);
    for (uint32_t t = 0; t < steps; ++t) {
        if (t % every == 0) {
            const size_t off = (size_t)(t / every) * n;
            ADJ_TRY(s, cudaMemcpyAsync(a.ckpt_x + off, s->x, bytes, cudaMemcpyDeviceToDevice, st));
            ADJ_TRY(s, cudaMemcpyAsync(a.ckpt_v + off, s->v, bytes, cudaMemcpyDeviceToDevice, st));
            if (nb)
                ADJ_TRY(s, cudaMemcpyAsync(a.ckpt_q + (size_t)(t / every) * nb, s->bodies.quat, nb * sizeof(float4),
                                           cudaMemcpyDeviceToDevice, st));
        }
        if (int rc = pbd_internal_enqueue_update(s, dt, st)) return rc;
    }
    a.recorded = true;
    a.version = s->version;
    a.dt = dt;
    a.steps = steps;
    a.every = every;
    a.nckpt = nck;
    return PBD_OK;
}

int pbd_record(pbd_system *s, float dt, uint32_t steps, uint32_t every, void *stream) {
    return pbd_rollout(s, dt, steps, every, stream);
}

int pbd_backward(pbd_system *s, const float *dL_dx, const float *dL_dv, float *dL_dx0, float *dL_dv0,
                 float *dL_dstiffness, void *stream) {
    if (int rc = pbd_internal_guard(s)) return rc;
    auto &a = s->adj;
    if (!a.recorded || a.version != s->version)
        return pbd_internal_fail(s, PBD_ERR_STATE, "no rollout to differentiate: call pbd_rollout after the last change of the scene");
    if (int rc = differentiable(s)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = s->n;
    const DevParams &P = s->dev;
    const bool batched = P.table != nullptr;
    const uint32_t iters = P.iterations;
    const size_t bytes = (size_t)n * sizeof(float4);
    const size_t per_step = 2u + 3u * iters;
    const uint64_t launches0 = s->launches, steps0 = s->steps;
    // work arrays
    size_t rec_have = a.rec_cap;
    ADJ_TRY(s, grow(&a.rec, rec_have, per_step * a.every * (size_t)n));
    a.rec_cap = rec_have;
    if (a.work_cap < s->cap) {
        for (float4 **p : {&a.gx, &a.gv, &a.gxo, &a.gt, &a.gy, &a.gu, &a.save_x, &a.save_v, &a.save_xo, &a.fl1, &a.fl2,
                           &a.w1, &a.w2, &a.w3}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
            ADJ_TRY(s, cudaMalloc((void **)p, (size_t)s->cap * sizeof(float4)));
        }
        if (a.cnt) cudaFree(a.cnt);
        if (a.lbar) cudaFree(a.lbar);
        a.cnt = nullptr;
        a.lbar = nullptr;
        ADJ_TRY(s, cudaMalloc((void **)&a.cnt, (size_t)s->cap * sizeof(uint32_t)));
        ADJ_TRY(s, cudaMalloc((void **)&a.lbar, (size_t)s->cap * sizeof(float)));
        a.work_cap = s->cap;
    }
    const uint32_t m = s->cons.m;
    if (m && a.stiff_cap < m) {
        if (a.gstiff) cudaFree(a.gstiff);
        a.gstiff = nullptr;
        ADJ_TRY(s, cudaMalloc((void **)&a.gstiff, (size_t)m * sizeof(float)));
        a.stiff_cap = m;
    }
    if (m) ADJ_TRY(s, cudaMemsetAsync(a.gstiff, 0, (size_t)m * sizeof(float), st));
    // the state after the rollout, restored at the end
    const uint32_t nbod = s->bodies.count;
    const size_t qbytes = (size_t)nbod * sizeof(float4);
    if (nbod)
        ADJ_TRY(s, cudaMemcpyAsync(a.ckpt_q + (size_t)a.nckpt * nbod, s->bodies.quat, qbytes, cudaMemcpyDeviceToDevice,
                                   st));
    ADJ_TRY(s, cudaMemcpyAsync(a.save_x, s->x, bytes, cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(s, cudaMemcpyAsync(a.save_v, s->v, bytes, cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(s, cudaMemcpyAsync(a.save_xo, s->x_old, bytes, cudaMemcpyDeviceToDevice, st));
    // incoming adjoints
    if (dL_dx) ADJ_TRY(s, cudaMemcpyAsync(a.gx, dL_dx, bytes, cudaMemcpyDeviceToDevice, st));
    else ADJ_TRY(s, cudaMemsetAsync(a.gx, 0, bytes, st));
    if (dL_dv) ADJ_TRY(s, cudaMemcpyAsync(a.gv, dL_dv, bytes, cudaMemcpyDeviceToDevice, st));
    else ADJ_TRY(s, cudaMemsetAsync(a.gv, 0, bytes, st));
    const bool contacts = s->n_contact != 0;
    const bool fluids = s->n_fluid != 0;
    const bool xsph = pbd_internal_any_xsph(s);
    const ConstraintBuffers &c = s->cons;
    const unsigned nb = blocks_for(n);
    const float dt = a.dt;
    const GridBuffers &g = s->grid;
#define ADJ_LAUNCH(KERNEL, GRID, ...)                                                     \
    do {                                                                                  \
        if (batched) KERNEL<true><<<(GRID), kBlock, 0, st>>>(__VA_ARGS__);                \
        else KERNEL<false><<<(GRID), kBlock, 0, st>>>(__VA_ARGS__);                       \
        ADJ_TRY(s, cudaGetLastError());                                                   \
    } while (0)
    for (int seg = (int)a.nckpt - 1; seg >= 0; --seg) {
        const uint32_t t0 = (uint32_t)seg * a.every;
        const uint32_t t1 = std::min(a.steps, t0 + a.every);
        // recompute the segment from its checkpoint, recording
        ADJ_TRY(s, cudaMemcpyAsync(s->x, a.ckpt_x + (size_t)seg * n, bytes, cudaMemcpyDeviceToDevice, st));
        ADJ_TRY(s, cudaMemcpyAsync(s->v, a.ckpt_v + (size_t)seg * n, bytes, cudaMemcpyDeviceToDevice, st));
        if (nbod)
            ADJ_TRY(s, cudaMemcpyAsync(s->bodies.quat, a.ckpt_q + (size_t)seg * nbod, qbytes, cudaMemcpyDeviceToDevice,
                                       st));
        for (uint32_t t = t0; t < t1; ++t)
            if (int rc = pbd_internal_enqueue_update(s, dt, st, a.rec + (t - t0) * per_step * n)) return rc;
        // reverse over its steps
        for (int t = (int)t1 - 1; t >= (int)t0; --t) {
            float4 *rec = a.rec + (size_t)(t - (int)t0) * per_step * n;
            const float4 *xfin = rec + (size_t)(1 + 3 * iters) * n;
            // x_old of this step for the friction and wall terms
            ADJ_TRY(s, cudaMemcpyAsync(s->x_old, rec, bytes, cudaMemcpyDeviceToDevice, st));
            if (xsph) {
                // XSPH over the last iteration's grid: gv (after XSPH) -> gv
                // (after the velocity update), w3 = its position part
                ADJ_TRY(s, cudaMemcpyAsync(s->x, rec + (size_t)(1 + 3 * (iters - 1)) * n, bytes,
                                           cudaMemcpyDeviceToDevice, st));
                if (int rc = pbd_internal_build_grid(s, st, false)) return rc;
                ADJ_LAUNCH(k_adj_vel_of, nb, P, n, dt, xfin, rec, a.w1);
                k_adj_gather_sorted<<<nb, kBlock, 0, st>>>(n, g.sorted_idx, a.w1, a.gv, a.w2, a.gu);
                ADJ_TRY(s, cudaGetLastError());
                ADJ_LAUNCH(k_adj_xsph, nb, P, n, g.sorted_x, g.sorted_attr, g.sorted_idx, g.cell_first, a.w2, a.gu,
                           a.gv, a.w3);
            }
            // gy <- adjoint of the final positions, gxo <- -gv / dt
            ADJ_LAUNCH(k_adj_velocity, nb, P, n, dt, a.gx, a.gv, a.gy, a.gxo);
            for (int it = (int)iters - 1; it >= 0; --it) {
                const uint32_t left = iters - 1u - (uint32_t)it;
                const float4 *xstart = rec + (size_t)(1 + 3 * it) * n;
                const float4 *ysolve = rec + (size_t)(2 + 3 * it) * n;
                const float4 *zdist = rec + (size_t)(3 + 3 * it) * n;
                // shape matching: gy (after shapes) -> gy (after pins)
                if (s->bodies.count) {
                    const BodyBuffers &bb = s->bodies;
                    ADJ_LAUNCH(k_adj_shapes, blocks_for(bb.count * 32u), P, left, bb.count, bb.range, bb.stiff, bb.rest,
                               zdist, a.gy);
                }
                // pins and distance constraints: gy (after pins) -> gt -> gy
                if (c.count) {
                    ADJ_TRY(s, cudaMemcpyAsync(a.gt, a.gy, bytes, cudaMemcpyDeviceToDevice, st));
                    const unsigned cb = blocks_for(c.count);
                    if (c.any_pin) ADJ_LAUNCH(k_adj_pins, cb, P, c.count, left, c.particle, c.pin, a.gt);
                    ADJ_TRY(s, cudaMemcpyAsync(a.gy, a.gt, bytes, cudaMemcpyDeviceToDevice, st));
                    if (c.any_distance) {
                        ADJ_LAUNCH(k_adj_distance, cb, P, c.count, left, c.particle, c.row, c.other, c.rest, c.stiff,
                                   c.occ_of, ysolve, a.gt, a.gy);
                        ADJ_LAUNCH(k_adj_stiffness, blocks_for(m), P, m, left, c.con_a, c.con_b, c.con_rest,
                                   c.con_stiff, c.occ_of, ysolve, a.gt, a.gstiff);
                    }
                }
                // contacts, fluid and walls: rebuild this iteration's grid,
                // recompute lambda, then prep (walls, u's adjoint, counts),
                // lambda's adjoint and the gather
                ADJ_TRY(s, cudaMemcpyAsync(s->x, xstart, bytes, cudaMemcpyDeviceToDevice, st));
                if (int rc = pbd_internal_build_grid(s, st, false)) return rc;
                if (fluids) ADJ_LAUNCH(k_adj_fluid_lambda, nb, P, n, g.sorted_x, g.sorted_attr, g.cell_first, a.fl1, a.fl2);
                ADJ_LAUNCH(k_adj_solve_prep, nb, P, n, left, contacts, fluids, g.sorted_x, g.sorted_attr, g.sorted_idx,
                           g.cell_first, s->x_old, a.fl1, a.fl2, a.gy, a.gu, a.cnt, a.gxo);
                if (fluids)
                    ADJ_LAUNCH(k_adj_fluid_lbar, nb, P, n, left, g.sorted_x, g.sorted_attr, g.cell_first, a.fl1, a.fl2,
                               a.gu, a.lbar);
#define ADJ_GATHER(BB, CC, FF)                                                                            \
    k_adj_solve_gather<BB, CC, FF><<<nb, kBlock, 0, st>>>(P, n, left, g.sorted_x, g.sorted_attr, g.sorted_idx,    \
                                                          g.cell_first, s->x_old, a.fl1, a.fl2, a.lbar, a.gu,    \
                                                          a.cnt, a.gy, a.gxo)
                if (batched) {
                    if (contacts && fluids) ADJ_GATHER(true, true, true);
                    else if (contacts) ADJ_GATHER(true, true, false);
                    else if (fluids) ADJ_GATHER(true, false, true);
                    else ADJ_GATHER(true, false, false);
                } else {
                    if (contacts && fluids) ADJ_GATHER(false, true, true);
                    else if (contacts) ADJ_GATHER(false, true, false);
                    else if (fluids) ADJ_GATHER(false, false, true);
                    else ADJ_GATHER(false, false, false);
                }
#undef ADJ_GATHER
                ADJ_TRY(s, cudaGetLastError());
                if (xsph && it == (int)iters - 1) {  // XSPH read this iteration's start positions
                    k_add4<<<nb, kBlock, 0, st>>>(n, a.gy, a.w3);
                    ADJ_TRY(s, cudaGetLastError());
                }
            }
            // predict: gy is now the adjoint of the predicted positions
            ADJ_LAUNCH(k_adj_predict, nb, P, n, dt, a.gy, a.gxo, a.gx, a.gv);
        }
    }
#undef ADJ_LAUNCH
    s->launches = launches0;  // the recomputation is not a user step
    s->steps = steps0;
    if (dL_dx0) ADJ_TRY(s, cudaMemcpyAsync(dL_dx0, a.gx, bytes, cudaMemcpyDeviceToDevice, st));
    if (dL_dv0) ADJ_TRY(s, cudaMemcpyAsync(dL_dv0, a.gv, bytes, cudaMemcpyDeviceToDevice, st));
    if (dL_dstiffness && m)
        ADJ_TRY(s, cudaMemcpyAsync(dL_dstiffness, a.gstiff, (size_t)m * sizeof(float), cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(s, cudaMemcpyAsync(s->x, a.save_x, bytes, cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(s, cudaMemcpyAsync(s->v, a.save_v, bytes, cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(s, cudaMemcpyAsync(s->x_old, a.save_xo, bytes, cudaMemcpyDeviceToDevice, st));
    if (nbod)
        ADJ_TRY(s, cudaMemcpyAsync(s->bodies.quat, a.ckpt_q + (size_t)a.nckpt * nbod, qbytes, cudaMemcpyDeviceToDevice,
                                   st));
    s->grid_valid = false;
    return PBD_OK;
}

}  // extern "C"
