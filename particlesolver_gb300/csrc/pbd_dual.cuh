// Forward-mode dual numbers and scalar-generic copies of the per-pair and
// per-particle projector formulas, for the adjoint kernels.
//
// Each projector's correction is written once here as a template over the
// scalar type T.  With T = float it is the forward formula; with T =
// Dual<N> seeded on N inputs it also carries d(correction)/d(input), i.e.
// a 3 x N block of the Jacobian, which the adjoint kernels contract with
// the incoming adjoint.  Branch decisions (contact on/off, static or
// kinetic friction, wall clamps, distance cut-off) follow the values, so
// they are the forward pass's decisions, held fixed as the derivative is
// taken.  The formulas follow the forward kernels in pbd_kernels.cu
// operation for operation (contact_delta, world_collide,
// k_distance_gather).
#pragma once

#include "pbd_device.cuh"

#if defined(__CUDACC__)

namespace pbd {

template <int N>
struct Dual {
    float v;
    float d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> dconst(float a) {
    Dual<N> r;
    r.v = a;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = 0.f;
    return r;
}

#define PBD_DUAL_BINOP(OP, VAL, DER)                                                      \
    template <int N>                                                                      \
    __device__ __forceinline__ Dual<N> operator OP(const Dual<N> &a, const Dual<N> &b) { \
        Dual<N> r;                                                                        \
        r.v = VAL;                                                                        \
        _Pragma("unroll") for (int k = 0; k < N; ++k) r.d[k] = DER;                      \
        return r;                                                                         \
    }
PBD_DUAL_BINOP(+, a.v + b.v, a.d[k] + b.d[k])
PBD_DUAL_BINOP(-, a.v - b.v, a.d[k] - b.d[k])
PBD_DUAL_BINOP(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
#undef PBD_DUAL_BINOP

template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) {
    Dual<N> r;
    r.v = a.v / b.v;
    const float ib = 1.f / b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N> &a) {
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, float b) {
    Dual<N> r = a;
    r.v = a.v + b;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(float a, const Dual<N> &b) { return b + a; }
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N> &a, float b) {
    Dual<N> r = a;
    r.v = a.v - b;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(float a, const Dual<N> &b) {
    Dual<N> r;
    r.v = a - b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -b.d[k];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, float b) {
    Dual<N> r;
    r.v = a.v * b;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(float a, const Dual<N> &b) { return b * a; }
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, float b) {
    Dual<N> r;
    r.v = a.v / b;
    const float ib = 1.f / b;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * ib;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(float a, const Dual<N> &b) { return dconst<N>(a) / b; }

// scalar helpers shared by float and Dual
__device__ __forceinline__ float val(float a) { return a; }
template <int N>
__device__ __forceinline__ float val(const Dual<N> &a) { return a.v; }

__device__ __forceinline__ float gsqrt(float a) { return sqrtf(a); }
template <int N>
__device__ __forceinline__ Dual<N> gsqrt(const Dual<N> &a) {
    Dual<N> r;
    r.v = sqrtf(a.v);
    const float h = (r.v > 0.f) ? 0.5f / r.v : 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
    return r;
}
__device__ __forceinline__ float grsqrt(float a) { return rsqrtf(a); }
template <int N>
__device__ __forceinline__ Dual<N> grsqrt(const Dual<N> &a) {
    Dual<N> r;
    r.v = rsqrtf(a.v);
    const float h = -0.5f * r.v / a.v;  // d(a^-1/2) = -1/2 a^-3/2
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
    return r;
}
// min / max with a constant: the derivative of the chosen branch
__device__ __forceinline__ float gmin(float a, float b) { return fminf(a, b); }
template <int N>
__device__ __forceinline__ Dual<N> gmin(const Dual<N> &a, float b) {
    return (a.v <= b) ? a : dconst<N>(b);
}
__device__ __forceinline__ float gmax(float a, float b) { return fmaxf(a, b); }
template <int N>
__device__ __forceinline__ Dual<N> gmax(const Dual<N> &a, float b) {
    return (a.v >= b) ? a : dconst<N>(b);
}
// a^n for a constant real n
__device__ __forceinline__ float gpow(float a, float n) { return powf(a, n); }
template <int N>
__device__ __forceinline__ Dual<N> gpow(const Dual<N> &a, float n) {
    Dual<N> r;
    r.v = powf(a.v, n);
    const float g = (a.v != 0.f) ? n * powf(a.v, n - 1.f) : 0.f;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
    return r;
}

template <class T>
struct V3 {
    T x, y, z;
};
template <class T>
__device__ __forceinline__ V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T>
__device__ __forceinline__ V3<T> operator+(const V3<T> &a, const V3<T> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T>
__device__ __forceinline__ V3<T> operator-(const V3<T> &a, const V3<T> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T, class S>
__device__ __forceinline__ V3<T> operator*(const V3<T> &a, const S &s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T, class S>
__device__ __forceinline__ V3<T> operator/(const V3<T> &a, const S &s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T>
__device__ __forceinline__ T gdot(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
__device__ __forceinline__ T glen(const V3<T> &a) { return gsqrt(gdot(a, a)); }

// Constants of scalar type T.
template <class T>
struct Scalar;
template <>
struct Scalar<float> {
    __device__ static float c(float a) { return a; }
};
template <int N>
struct Scalar<Dual<N>> {
    __device__ static Dual<N> c(float a) { return dconst<N>(a); }
};
template <class T>
__device__ __forceinline__ T cst(float a) { return Scalar<T>::c(a); }
template <class T>
__device__ __forceinline__ V3<T> lift(float3 a) { return {cst<T>(a.x), cst<T>(a.y), cst<T>(a.z)}; }

// A float3 as the dual variables first, first + 1, first + 2.
template <int N>
__device__ __forceinline__ V3<Dual<N>> seed(float3 a, int first) {
    V3<Dual<N>> r{dconst<N>(a.x), dconst<N>(a.y), dconst<N>(a.z)};
    r.x.d[first] = 1.f;
    r.y.d[first + 1] = 1.f;
    r.z.d[first + 2] = 1.f;
    return r;
}

// g . d(r)/d(variables first .. first + 2): one 3x3 Jacobian block
// contracted with the incoming adjoint g.
template <int N>
__device__ __forceinline__ float3 contract(const V3<Dual<N>> &r, float3 g, int first) {
    return make_float3(g.x * r.x.d[first] + g.y * r.y.d[first] + g.z * r.z.d[first],
                       g.x * r.x.d[first + 1] + g.y * r.y.d[first + 1] + g.z * r.z.d[first + 1],
                       g.x * r.x.d[first + 2] + g.y * r.y.d[first + 2] + g.z * r.z.d[first + 2]);
}

// One contact pair's contribution to particle i's correction (one term of
// contact_delta): separation to 2.001 r shared by inverse mass, divided by
// i's contact count n_i, plus static / kinetic friction for solid pairs
// against the start-of-step positions prev_i, prev_j (the reference's
// (prev_i + dp2 - prev_j) term included as written).
template <class T>
__device__ __forceinline__ V3<T> contact_pair(const DevParams &P, V3<T> pi, float wi, int phi, V3<T> previ, V3<T> pj,
                                              float wj, int phj, V3<T> prevj, float fnb) {
    V3<T> out = lift<T>(make_float3(0.f, 0.f, 0.f));
    const V3<T> diff = pi - pj;
    const T dist = glen(diff);
    const T mag = dist - P.collide_dist;
    const float colw = wi, colw2 = wj;
    const float wsum = colw + colw2;
    if (wsum == 0.f || val(dist) == 0.f) return out;
    const T scale = mag / wsum;
    const V3<T> dp = diff * (scale / dist);
    const V3<T> dp1 = (dp * (-colw)) / fnb;
    const V3<T> dp2 = (dp * colw2) / fnb;
    out = dp1;
    if (phi < kSolid || phj < kSolid) return out;
    const V3<T> nf = diff * grsqrt(gdot(diff, diff));
    const V3<T> dprel = (pi + dp1 - previ) - (previ + dp2 - prevj);
    const V3<T> dpt = dprel - nf * gdot(dprel, nf);
    const T ldpt = glen(dpt);
    if (val(ldpt) < kEps) return out;
    if (val(ldpt) < P.cs * val(dist)) out = out - (dpt * colw) / wsum;
    else out = out - dpt * gmin((dist * P.ck) / ldpt, 1.f);
    return out;
}

// collide_world_functor as in world_collide: clamps (constant after the
// clamp) and wall friction against prev for phases >= CLOTH.
template <class T>
__device__ __forceinline__ V3<T> world_generic(const DevParams &P, V3<T> e, int phase, V3<T> pos) {
    const float d = P.r;
    float eps = (phase < kSolid) ? d * 0.01f : d * 0.f;
    float3 nrm = make_float3(0.f, 0.f, 0.f);
    const bool twod = (P.flags & kFlagTwoD) != 0u;
    if (val(e.y) < P.bmin.y + P.r) {
        e.y = cst<T>(P.bmin.y + P.r + P.rands[5] * eps);
        nrm.y += 1.f;
    }
    eps = d * 0.01f;
    if (val(e.x) > P.bmax.x - P.r) {
        e.x = cst<T>(P.bmax.x - (P.r + P.rands[0] * eps));
        nrm.x += -1.f;
    }
    if (val(e.x) < P.bmin.x + P.r) {
        e.x = cst<T>(P.bmin.x + (P.r + P.rands[1] * eps));
        nrm.x += 1.f;
    }
    if (val(e.y) > P.bmax.y - P.r) {
        e.y = cst<T>(P.bmax.y - (P.r + P.rands[2] * eps));
        nrm.y += -1.f;
    }
    if (!twod) {
        if (val(e.z) > P.bmax.z - P.r) {
            e.z = cst<T>(P.bmax.z - (P.r + P.rands[3] * eps));
            nrm.z += -1.f;
        }
        if (val(e.z) < P.bmin.z + P.r) {
            e.z = cst<T>(P.bmin.z + (P.r + P.rands[4] * eps));
            nrm.z += 1.f;
        }
    } else {
        e.z = cst<T>(P.twod_z);
    }
    if (len3(nrm) < kEps || phase < kCloth) return e;
    if (twod) pos.z = cst<T>(P.twod_z);
    const V3<T> dp = e - pos;
    const V3<T> n = lift<T>(nrm);
    const V3<T> dpt = dp - n * gdot(dp, n);
    const T ldpt = glen(dpt);
    if (val(ldpt) < kEps) return e;
    if (val(ldpt) < P.ws * d) return e - dpt;
    return e - dpt * gmin((P.wk * d) / ldpt, 1.f);
}

// One distance-constraint incidence's correction of x_k before the
// division by k's constraint count (k_distance_gather).
template <class T>
__device__ __forceinline__ V3<T> distance_term(const DevParams &P, V3<T> xk, float wk, V3<T> xo, float wo, float rest,
                                               T stiff) {
    const V3<T> rel = xk - xo;
    const T dist = glen(rel);
    if (!(val(dist) > kMinDistLen)) return lift<T>(make_float3(0.f, 0.f, 0.f));
    T mag;
    if (P.flags & kFlagDistanceMassWeighted) {
        const float ws = wk + wo;
        mag = (ws > 0.f) ? (rest - dist) * (wk / ws) : cst<T>(0.f);
    } else {
        mag = (rest - dist) * .5f;
    }
    return (rel / dist) * (mag * stiff);
}

// ----------------------------------------------------------------- PBF

// One neighbour's terms of the lambda pass (LambdaAcc::add): its poly6
// density term and its spiky gradient over rho0 (zero below the 1e-4
// length cut-off).  mass_factor: 1 / w_i, or 1 / w_j with
// PBD_FLAG_DENSITY_NEIGHBOR_MASS.
template <class T>
struct LambdaTerm {
    T ro;
    V3<T> sg;
};

template <class T>
__device__ __forceinline__ LambdaTerm<T> lambda_term(const DevParams &P, V3<T> pi, V3<T> pj, float mass_factor,
                                                     float spiky_r) {
    const V3<T> dr = pi - pj;
    const T d2 = gdot(dr, dr);
    const T hm2 = P.h2 - d2;
    LambdaTerm<T> t;
    t.ro = hm2 * hm2 * hm2 * (P.poly6 * mass_factor);
    const T rs = grsqrt(gmax(d2, kMinSpiky2));
    const T hm = P.h - d2 * rs;
    if (val(d2) >= kMinSpiky2) t.sg = dr * (hm * hm * rs * spiky_r);
    else t.sg = lift<T>(make_float3(0.f, 0.f, 0.f));
    return t;
}

// lambda from the pass's sums: ro (neighbour terms, own term added here),
// denom = sum |sg|^2 and grad = -sum sg.
template <class T>
__device__ __forceinline__ T lambda_of(const DevParams &P, T ro, T denom, V3<T> grad, float inv_w, float inv_rho0) {
    const T r = ro + P.poly6_self * inv_w;
    return -(r * inv_rho0 - 1.f) / (denom + gdot(grad, grad) + P.relax);
}

// s_corr ratio^n (scorr_pow).
template <class T>
__device__ __forceinline__ T scorr_pow_g(const DevParams &P, T ratio) {
    if (P.scorr_n_int == 4) {
        const T r2 = ratio * ratio;
        return r2 * r2;
    }
    if (P.scorr_n_int > 0) {
        T r = ratio;
        for (int k = 1; k < P.scorr_n_int; ++k) r = r * ratio;
        return r;
    }
    return gpow(ratio, P.scorr_n);
}

// One neighbour's term of the delta pass (delta_add) before the division
// by rho0 + n: (lambda_i + lambda_j + s_corr) times the spiky gradient,
// with the reference's (0, EPS, 0) direction below the cut-off.
template <class T>
__device__ __forceinline__ V3<T> delta_term(const DevParams &P, V3<T> pi, V3<T> pj, T lam_sum, float poly6_ref) {
    const V3<T> dr = pi - pj;
    const T d2 = gdot(dr, dr);
    const T hm2 = P.h2 - d2;
    const T coef = lam_sum - P.scorr_k * scorr_pow_g<T>(P, hm2 * hm2 * hm2 * poly6_ref);
    if (val(d2) >= kMinSpiky2) {
        const T rs = grsqrt(d2);
        const T hm = P.h - d2 * rs;
        return dr * (coef * (-P.spiky) * hm * hm * rs);
    }
    const T hz = P.h - gsqrt(d2);
    V3<T> out = lift<T>(make_float3(0.f, 0.f, 0.f));
    out.y = coef * (-P.spiky * kEps) * hz * hz;
    return out;
}

}  // namespace pbd

#endif  // __CUDACC__
