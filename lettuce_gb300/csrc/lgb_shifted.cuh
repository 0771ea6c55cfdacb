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
// f32x2 instructions of sm_100+). Both give bit-identical per-cell results
// because every operation is an explicit round-to-nearest intrinsic (the
// reciprocal of the density: one approximate instruction, the same in both)
// AND no
// product is ever an operand of an add or subtract: the compiler fuses a
// packed multiply into a following packed add (the scalar __fmul_rn is never
// fused), so every multiply-add here is written as an explicit FMA, and the
// equilibrium is expressed through e.j and j.j so that no rounded product of
// 1/rho feeds a sum.
#pragma once

#include <cuda_runtime.h>

#include "lgb_collide.cuh"

namespace lgb {

// 1 / rho on one- and two-dimensional stencils: the hardware's approximate
// reciprocal (__fdividef, within 2 ulp; the same instruction in both lane
// types, so they stay bit-identical) (1), or the correctly rounded
// __frcp_rn (0); three-dimensional stencils always take __frcp_rn. Far
// below the 16-bit storage's rounding either way. Measured: the batched
// D2Q9 fp16 TRT step 147.1k -> 150.9k MLUPS; the D3Q19 two-cell kernels
// lost with it (pull 82.6k -> 81.1k, AA pair 76.6k -> 71.8k: the AA odd
// step spilled 208 bytes instead of 40).
#ifndef LGB_SHIFTED_FAST_RCP_2D
#define LGB_SHIFTED_FAST_RCP_2D 1
#endif
__device__ __forceinline__ float shifted_rcp(float a, bool fast) {
    return fast ? __fdividef(1.0f, a) : __frcp_rn(a);
}

struct Lane1 {
    using V = float;
    static __device__ __forceinline__ V set(float a) { return a; }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ V rcp(V a, bool fast) { return shifted_rcp(a, fast); }
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
    static __device__ __forceinline__ V rcp(V a, bool fast) {
        return make_float2(shifted_rcp(a.x, fast), shifted_rcp(a.y, fast));
    }
};

// density deviation, density, 1/density and momentum of shifted populations
template <class S, class L>
__device__ __forceinline__ void shifted_moments(const typename L::V (&h)[S::Q], typename L::V &drho,
                                                typename L::V &rho, typename L::V &inv,
                                                typename L::V (&j)[3]) {
    using V = typename L::V;
    V r = h[0];
#pragma unroll
    for (int q = 1; q < S::Q; ++q) r = L::add(r, h[q]);
    drho = r;
    rho = L::add(r, L::set(1.0f));
    inv = L::rcp(rho, LGB_SHIFTED_FAST_RCP_2D && S::D < 3);
#pragma unroll
    for (int d = 0; d < 3; ++d) j[d] = L::set(0.0f);
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        V acc = L::set(0.0f);
        bool first = true;
#pragma unroll
        for (int q = 1; q < S::Q; ++q) {
            const int c = S::e(q, d);
            if (c == 0) continue;
            if (first) { acc = c > 0 ? h[q] : L::sub(L::set(0.0f), h[q]); first = false; }
            else acc = c > 0 ? L::add(acc, h[q]) : L::sub(acc, h[q]);
        }
        j[d] = acc;
    }
}

// e_q . x for a compile-time q (sums and differences only)
template <class S, class L>
__device__ __forceinline__ typename L::V dot_e(int q, const typename L::V (&x)[3]) {
    using V = typename L::V;
    V r = L::set(0.0f);
    bool first = true;
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        const int c = S::e(q, d);
        if (c == 0) continue;
        if (first) { r = c > 0 ? x[d] : L::sub(L::set(0.0f), x[d]); first = false; }
        else r = c > 0 ? L::add(r, x[d]) : L::sub(r, x[d]);
    }
    return r;
}

template <class S, class L, int COLL>
__device__ __forceinline__ void collide_shifted(typename L::V (&h)[S::Q], const CollideParams &cp) {
    using V = typename L::V;
    if constexpr (COLL == LGB_NO_COLLISION) {
        return;
    } else {
        // With ej = e_q . j and e.u = ej / rho the shifted equilibrium is
        //   heq_q = w_q X_q,  X_q = base + 3 ej + 4.5 ej^2 / rho,
        //   base = drho - 1.5 (j.j) / rho,
        // and the opposite direction has X_o = base - 3 ej + 4.5 ej^2 / rho.
        V drho, rho, inv, j[3];
        shifted_moments<S, L>(h, drho, rho, inv, j);
        V jj = L::mul(j[0], j[0]);
#pragma unroll
        for (int d = 1; d < S::D; ++d) jj = L::fma(j[d], j[d], jj);
        const V base = L::fma(jj, L::mul(inv, L::set(-1.5f)), drho);
        const V k45 = L::mul(inv, L::set(4.5f));
        if constexpr (COLL == LGB_BGK) {
            // h' = (1 - omega) h + (omega w_q) X_q
            const float om = cp.f_omega;
            const V om1 = L::set(cp.f_one_minus_omega);
            h[0] = L::fma(L::set(om * (float)S::w(0)), base, L::mul(om1, h[0]));
#pragma unroll
            for (int q = 1; q < S::Q; ++q) {
                const int o = S::opp(q);
                if (o < q) continue;
                const V ow = L::set(om * (float)S::w(q));
                const V ej = dot_e<S, L>(q, j);
                const V sq = L::fma(L::mul(ej, k45), ej, base);
                h[q] = L::fma(ow, L::fma(ej, L::set(3.0f), sq), L::mul(om1, h[q]));
                h[o] = L::fma(ow, L::fma(ej, L::set(-3.0f), sq), L::mul(om1, h[o]));
            }
        } else {
            // TRT: with heq_q + heq_o = 2 w s and heq_q - heq_o = 6 w ej,
            //   dp = (h_q + h_o) - 2 w s,  dm = (h_q - h_o) - 6 w ej,
            //   h_q' = h_q - dp / (2 tau+) - dm / (2 tau-),
            //   h_o' = h_o - dp / (2 tau+) + dm / (2 tau-)
            const V nap = L::set(-cp.f_inv_2tp);
            const V am = L::set(cp.f_inv_2tm), nam = L::set(-cp.f_inv_2tm);
            {
                const V dp = L::fma(L::set(-2.0f * (float)S::w(0)), base, L::add(h[0], h[0]));
                h[0] = L::fma(nap, dp, h[0]);
            }
#pragma unroll
            for (int q = 1; q < S::Q; ++q) {
                const int o = S::opp(q);
                if (o < q) continue;
                const float w = (float)S::w(q);
                const V ej = dot_e<S, L>(q, j);
                const V sq = L::fma(L::mul(ej, k45), ej, base);
                const V dp = L::fma(L::set(-2.0f * w), sq, L::add(h[q], h[o]));
                const V dm = L::fma(L::set(-6.0f * w), ej, L::sub(h[q], h[o]));
                h[q] = L::fma(nap, dp, L::fma(nam, dm, h[q]));
                h[o] = L::fma(nap, dp, L::fma(am, dm, h[o]));
            }
        }
    }
}

// collisions computed in shifted space (16-bit storage, unmasked)
template <int COLL> __host__ __device__ constexpr bool shifted_collision() {
    return COLL == LGB_NO_COLLISION || COLL == LGB_BGK || COLL == LGB_TRT;
}

}  // namespace lgb
