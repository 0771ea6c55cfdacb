// Per-cell moments, equilibrium and collision operators on a register array
// f[Q] in the compute type R.
//
//   moments      lettuce/_flow.py:157-193
//   equilibrium  lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24
//                (w rho (1 + e.u/cs^2 + (e.u)^2/(2 cs^4) - u.u/(2 cs^2)),
//                cs^2 = 1/3, evaluated in the expanded form below)
//   BGK          lettuce/ext/_collision/bgk_collision.py:17-22
//   TRT          lettuce/ext/_collision/trt_collision.py:16-27
//   KBC          lettuce/ext/_collision/kbc_collision.py:22-160
#pragma once

#include "lgb_stencil.cuh"

namespace lgb {

template <class S, class R>
LGB_HD void cell_moments(const R (&f)[S::Q], R &rho, R (&u)[3]) {
    R r = R(0);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) r += f[q];
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        R j = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) {
            const int c = S::e(q, d);
            if (c == 1) j += f[q];
            else if (c == -1) j -= f[q];
        }
        u[d] = j;
    }
    const R inv = R(1) / r;
#pragma unroll
    for (int d = 0; d < S::D; ++d) u[d] *= inv;
    rho = r;
}

template <class S, class R>
LGB_HD R feq_q(int q, R rho, const R (&u)[3], R uu) {
    R eu = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        const int c = S::e(q, d);
        if (c == 1) eu += u[d];
        else if (c == -1) eu -= u[d];
    }
    const R a = R(3) * eu;
    return R(S::w(q)) * rho * (R(1) + a + R(0.5) * a * a - R(1.5) * uu);
}

template <class S, class R>
LGB_HD R dot_uu(const R (&u)[3]) {
    R uu = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) uu += u[d] * u[d];
    return uu;
}

template <class S, class R>
LGB_HD void set_equilibrium(R (&f)[S::Q], R rho, const R (&u)[3]) {
    const R uu = dot_uu<S>(u);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = feq_q<S>(q, rho, u, uu);
}

struct CollideParams {
    double omega;        // 1 / tau (BGK)
    double inv_2tp;      // 1 / (2 tau_plus) (TRT)
    double inv_2tm;      // 1 / (2 tau_minus) (TRT)
    double beta;         // 1 / (2 tau) (KBC)
};

template <class S, class R>
LGB_HD void collide_bgk(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    cell_moments<S>(f, rho, u);
    const R uu = dot_uu<S>(u);
    const R om = R(cp.omega);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = f[q] - om * (f[q] - feq_q<S>(q, rho, u, uu));
    rho_out = rho;
}

template <class S, class R>
LGB_HD void collide_trt(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    cell_moments<S>(f, rho, u);
    const R uu = dot_uu<S>(u);
    const R ap = R(cp.inv_2tp), am = R(cp.inv_2tm);
    R out[S::Q];
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        const int o = S::opp(q);
        const R eq = feq_q<S>(q, rho, u, uu), eo = feq_q<S>(o, rho, u, uu);
        const R dp = (f[q] + f[o]) - (eq + eo);
        const R dm = (f[q] - f[o]) - (eq - eo);
        out[q] = f[q] - dp * ap - dm * am;
    }
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = out[q];
    rho_out = rho;
}

// KBC shear part s_q of a population set g (with density rho_g): the
// moment transform of kbc_collision.py:25-39 restricted to the second
// moments it consumes, and compute_s_seq_from_m_{3d,2d} (:44-94).
template <class S, class R>
LGB_HD void kbc_shear(const R (&g)[S::Q], R rho_g, R (&s)[S::Q]) {
    static_assert(S::Q == 27 || S::Q == 9, "KBC is defined for D3Q27 and D2Q9");
    if constexpr (S::Q == 27) {
        R mxx = 0, myy = 0, mzz = 0, mxy = 0, mxz = 0, myz = 0;
#pragma unroll
        for (int q = 0; q < 27; ++q) {
            const int ex = S::e(q, 0), ey = S::e(q, 1), ez = S::e(q, 2);
            if (ex) mxx += g[q];
            if (ey) myy += g[q];
            if (ez) mzz += g[q];
            if (ex * ey == 1) mxy += g[q]; else if (ex * ey == -1) mxy -= g[q];
            if (ex * ez == 1) mxz += g[q]; else if (ex * ez == -1) mxz -= g[q];
            if (ey * ez == 1) myz += g[q]; else if (ey * ez == -1) myz -= g[q];
        }
        const R inv = R(1) / rho_g;
        mxx *= inv; myy *= inv; mzz *= inv; mxy *= inv; mxz *= inv; myz *= inv;
        const R T = mxx + myy + mzz, Nxz = mxx - mzz, Nyz = myy - mzz;
        const R r6 = R(1.0 / 6.0) * rho_g, r4 = R(0.25) * rho_g;
#pragma unroll
        for (int q = 0; q < 27; ++q) s[q] = R(0);
        s[0] = rho_g * -T;
        s[1] = s[2] = r6 * (R(2) * Nxz - Nyz + T);
        s[3] = s[4] = r6 * (R(2) * Nyz - Nxz + T);
        s[5] = s[6] = r6 * (-Nxz - Nyz + T);
        s[7] = s[8] = r4 * myz;
        s[9] = s[10] = -r4 * myz;
        s[11] = s[12] = r4 * mxz;
        s[13] = s[14] = -r4 * mxz;
        s[15] = s[16] = r4 * mxy;
        s[17] = s[18] = -r4 * mxy;
    } else {
        R mxx = 0, myy = 0, mxy = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int ex = S::e(q, 0), ey = S::e(q, 1);
            if (ex) mxx += g[q];
            if (ey) myy += g[q];
            if (ex * ey == 1) mxy += g[q]; else if (ex * ey == -1) mxy -= g[q];
        }
        const R inv = R(1) / rho_g;
        mxx *= inv; myy *= inv; mxy *= inv;
        const R T = mxx + myy, Nn = mxx - myy;
        s[0] = rho_g * -T;
        s[1] = s[3] = R(0.5) * rho_g * (R(0.5) * (T + Nn));
        s[2] = s[4] = R(0.5) * rho_g * (R(0.5) * (T - Nn));
        s[5] = s[7] = R(0.25) * rho_g * mxy;
        s[6] = s[8] = -s[5];
    }
}

template <class S, class R>
LGB_HD void collide_kbc(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    cell_moments<S>(f, rho, u);
    const R uu = dot_uu<S>(u);
    R feq[S::Q];
    R rho_eq = R(0);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) { feq[q] = feq_q<S>(q, rho, u, uu); rho_eq += feq[q]; }
    R ds[S::Q], t[S::Q];
    kbc_shear<S>(f, rho, ds);
    kbc_shear<S>(feq, rho_eq, t);
    R sum_s = R(0), sum_h = R(0);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        ds[q] -= t[q];
        const R dh = f[q] - feq[q] - ds[q];
        const R ifeq = R(1) / feq[q];
        sum_s += ds[q] * dh * ifeq;
        sum_h += dh * dh * ifeq;
        t[q] = dh;
    }
    const R beta = R(cp.beta);
    const R ib = R(1) / beta;
    R gamma = ib - (R(2) - ib) * sum_s / sum_h;
    // kbc_collision.py:155-158: gamma < 1e-15 or NaN -> 2
    if (!(gamma >= R(1e-15))) gamma = R(2);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = f[q] - beta * (R(2) * ds[q] + gamma * t[q]);
    rho_out = rho;
}

template <int COLL, class S, class R>
LGB_HD void collide(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    if constexpr (COLL == LGB_BGK) {
        collide_bgk<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_TRT) {
        collide_trt<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_KBC) {
        collide_kbc<S>(f, cp, rho_out);
    } else {
        R r = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) r += f[q];
        rho_out = r;
    }
}

}  // namespace lgb
