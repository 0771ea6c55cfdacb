// Collision arithmetic on shifted populations h_q = f_q - w_q, used for the
// 16-bit storage formats (BGK, TRT and no collision). With sum_q w_q = 1 and
// sum_q w_q e_q = 0 the moments and the equilibrium stay small quantities:
//   drho = sum_q h_q,  rho = 1 + drho,  j = sum_q e_q h_q,  u = j / rho
//   heq_q = feq_q - w_q = w_q (drho + rho (3 e.u + 9/2 (e.u)^2 - 3/2 u.u))
// and BGK / TRT act on h exactly as on f because w_q = w_opposite(q)
// (lettuce/ext/_collision/bgk_collision.py:17-22, trt_collision.py:16-27).
//
// The arithmetic is written once over a lane type L: L = Lane1 (one cell per
// thread, float) or Lane2 (two cells per thread, float2 with the packed
// f32x2 instructions of sm_100+). Every operation is an explicit
// round-to-nearest intrinsic, so both give bit-identical per-cell results.
#pragma once

#include <cuda_runtime.h>

#include "lgb_collide.cuh"

namespace lgb {

struct Lane1 {
    using V = float;
    static __device__ __forceinline__ V set(float a) { return a; }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ V rcp(V a) { return __frcp_rn(a); }
};

struct Lane2 {
    using V = float2;
    static __device__ __forceinline__ V set(float a) { return make_float2(a, a); }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) {
        return __fadd2_rn(a, make_float2(-b.x, -b.y));
    }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
    static __device__ __forceinline__ V rcp(V a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
};

// density deviation, density and velocity of shifted populations
template <class S, class L>
__device__ __forceinline__ void shifted_moments(const typename L::V (&h)[S::Q], typename L::V &drho,
                                                typename L::V &rho, typename L::V (&u)[3]) {
    using V = typename L::V;
    V r = h[0];
#pragma unroll
    for (int q = 1; q < S::Q; ++q) r = L::add(r, h[q]);
    drho = r;
    rho = L::add(r, L::set(1.0f));
    const V inv = L::rcp(rho);
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = L::set(0.0f);
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        V j = L::set(0.0f);
        bool first = true;
#pragma unroll
        for (int q = 1; q < S::Q; ++q) {
            const int c = S::e(q, d);
            if (c == 0) continue;
            if (first) { j = c > 0 ? h[q] : L::sub(L::set(0.0f), h[q]); first = false; }
            else j = c > 0 ? L::add(j, h[q]) : L::sub(j, h[q]);
        }
        u[d] = L::mul(j, inv);
    }
}

// e_q . u for a compile-time q
template <class S, class L>
__device__ __forceinline__ typename L::V dot_e_u(int q, const typename L::V (&u)[3]) {
    using V = typename L::V;
    V eu = L::set(0.0f);
    bool first = true;
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        const int c = S::e(q, d);
        if (c == 0) continue;
        if (first) { eu = c > 0 ? u[d] : L::sub(L::set(0.0f), u[d]); first = false; }
        else eu = c > 0 ? L::add(eu, u[d]) : L::sub(eu, u[d]);
    }
    return eu;
}

// weight class of a velocity: |e|^2 (0 rest, 1 axis, 2 face diagonal,
// 3 space diagonal); every lettuce stencil has one weight per class
template <class S> __host__ __device__ constexpr int weight_class(int q) {
    int s = 0;
    for (int d = 0; d < S::D; ++d) s += S::e(q, d) * S::e(q, d);
    return s;
}
// first velocity of class k, or -1 when the stencil has none
template <class S> __host__ __device__ constexpr int weight_class_rep(int k) {
    for (int q = 0; q < S::Q; ++q)
        if (weight_class<S>(q) == k) return q;
    return -1;
}

// shifted equilibria of the pair (q, opposite(q)): they share e.u up to sign
template <class S, class L>
__device__ __forceinline__ void shifted_feq_pair(int q, typename L::V drho, typename L::V rho,
                                                 const typename L::V (&u)[3], typename L::V c,
                                                 typename L::V &heq_q, typename L::V &heq_o) {
    using V = typename L::V;
    const V a = L::mul(dot_e_u<S, L>(q, u), L::set(3.0f));
    const V b = L::fma(L::mul(a, L::set(0.5f)), a, c);  // c = -1.5 u.u
    const V wq = L::set((float)S::w(q));
    heq_q = L::mul(wq, L::fma(rho, L::add(b, a), drho));
    heq_o = L::mul(wq, L::fma(rho, L::sub(b, a), drho));
}

template <class S, class L, int COLL>
__device__ __forceinline__ void collide_shifted(typename L::V (&h)[S::Q], const CollideParams &cp) {
    using V = typename L::V;
    if constexpr (COLL == LGB_NO_COLLISION) {
        return;
    } else {
        V drho, rho, u[3];
        shifted_moments<S, L>(h, drho, rho, u);
        V uu = L::mul(u[0], u[0]);
#pragma unroll
        for (int d = 1; d < S::D; ++d) uu = L::fma(u[d], u[d], uu);
        const V c = L::mul(uu, L::set(-1.5f));
        if constexpr (COLL == LGB_BGK) {
            // h' = (1 - w) h + omega heq with omega folded into the
            // per-weight-class factors omega w rho and omega w drho:
            //   omega heq_q = omega w rho (b +- 3 e.u) + omega w drho,
            //   b = 4.5 (e.u)^2 - 1.5 u.u
            const V om1 = L::set((float)(1.0 - cp.omega));
            const V omr = L::mul(L::set((float)cp.omega), rho);
            const V omd = L::mul(L::set((float)cp.omega), drho);
            V wr[4], wd[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int q = weight_class_rep<S>(k);
                if (q < 0) continue;
                wr[k] = L::mul(omr, L::set((float)S::w(q)));
                wd[k] = L::mul(omd, L::set((float)S::w(q)));
            }
            h[0] = L::fma(om1, h[0], L::fma(wr[0], c, wd[0]));
#pragma unroll
            for (int q = 1; q < S::Q; ++q) {
                const int o = S::opp(q);
                if (o < q) continue;
                const int k = weight_class<S>(q);
                const V eu = dot_e_u<S, L>(q, u);
                const V b = L::fma(L::mul(eu, L::set(4.5f)), eu, c);
                const V p = L::fma(eu, L::set(3.0f), b);
                const V m = L::fma(eu, L::set(-3.0f), b);
                h[q] = L::fma(om1, h[q], L::fma(wr[k], p, wd[k]));
                h[o] = L::fma(om1, h[o], L::fma(wr[k], m, wd[k]));
            }
        } else {  // TRT
            const V ap = L::set((float)cp.inv_2tp), am = L::set((float)cp.inv_2tm);
            {
                V e0, dummy;
                shifted_feq_pair<S, L>(0, drho, rho, u, c, e0, dummy);
                const V dp = L::sub(L::add(h[0], h[0]), L::add(e0, e0));
                h[0] = L::sub(h[0], L::mul(dp, ap));
            }
#pragma unroll
            for (int q = 1; q < S::Q; ++q) {
                const int o = S::opp(q);
                if (o < q) continue;
                V eq, eo;
                shifted_feq_pair<S, L>(q, drho, rho, u, c, eq, eo);
                const V dp = L::sub(L::add(h[q], h[o]), L::add(eq, eo));
                const V dm = L::sub(L::sub(h[q], h[o]), L::sub(eq, eo));
                const V sp = L::mul(dp, ap), sm = L::mul(dm, am);
                h[q] = L::sub(L::sub(h[q], sp), sm);
                h[o] = L::add(L::sub(h[o], sp), sm);
            }
        }
    }
}

// collisions computed in shifted space (16-bit storage, unmasked)
template <int COLL> __host__ __device__ constexpr bool shifted_collision() {
    return COLL == LGB_NO_COLLISION || COLL == LGB_BGK || COLL == LGB_TRT;
}

}  // namespace lgb
