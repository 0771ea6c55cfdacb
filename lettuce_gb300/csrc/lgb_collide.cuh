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

// reciprocal used by the KBC entropy sums: the hardware approximation in
// float32 (2 ulp), exact division in float64
LGB_HD float kbc_rcp(float x) {
#ifdef __CUDA_ARCH__
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}
LGB_HD double kbc_rcp(double x) { return 1.0 / x; }

// Entropic KBC collision (lettuce/ext/_collision/kbc_collision.py:96-160),
// D3Q27 and D2Q9. The shear part delta_s = s(f) - s(feq) is linear in the
// second moments, s(.) of kbc_collision.py:44-94; for the quadratic
// equilibrium those moments are rho (delta_ab / 3 + u_a u_b) exactly (and
// sum_q feq_q = rho), so delta_s is formed from the deviations
// d_ab = m_ab(f) / rho - (delta_ab / 3 + u_a u_b). Then
//   delta_h = f - feq - delta_s,
//   gamma = 1/beta - (2 - 1/beta) <delta_s delta_h / feq> / <delta_h^2 / feq>
// (2 where that is below 1e-15 or NaN) and f <- f - beta (2 delta_s + gamma delta_h).
template <class S, class R>
LGB_HD void collide_kbc(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    static_assert(S::Q == 27 || S::Q == 9, "KBC is defined for D3Q27 and D2Q9");
    R rho, u[3];
    cell_moments<S>(f, rho, u);
    const R uu = dot_uu<S>(u);
    const R inv_rho = R(1) / rho;
    const R third = R(1.0 / 3.0);
    // delta_s by velocity class (index into ds_val below)
    R ds_val[8];
    if constexpr (S::Q == 27) {
        R mxx = 0, myy = 0, mzz = 0, mxy = 0, mxz = 0, myz = 0;
#pragma unroll
        for (int q = 0; q < 27; ++q) {
            const int ex = S::e(q, 0), ey = S::e(q, 1), ez = S::e(q, 2);
            if (ex) mxx += f[q];
            if (ey) myy += f[q];
            if (ez) mzz += f[q];
            if (ex * ey == 1) mxy += f[q]; else if (ex * ey == -1) mxy -= f[q];
            if (ex * ez == 1) mxz += f[q]; else if (ex * ez == -1) mxz -= f[q];
            if (ey * ez == 1) myz += f[q]; else if (ey * ez == -1) myz -= f[q];
        }
        const R dxx = mxx * inv_rho - (third + u[0] * u[0]);
        const R dyy = myy * inv_rho - (third + u[1] * u[1]);
        const R dzz = mzz * inv_rho - (third + u[2] * u[2]);
        const R dxy = mxy * inv_rho - u[0] * u[1];
        const R dxz = mxz * inv_rho - u[0] * u[2];
        const R dyz = myz * inv_rho - u[1] * u[2];
        const R dT = dxx + dyy + dzz, dNxz = dxx - dzz, dNyz = dyy - dzz;
        const R r6 = R(1.0 / 6.0) * rho, r4 = R(0.25) * rho;
        ds_val[0] = rho * -dT;
        ds_val[1] = r6 * (R(2) * dNxz - dNyz + dT);
        ds_val[2] = r6 * (R(2) * dNyz - dNxz + dT);
        ds_val[3] = r6 * (-dNxz - dNyz + dT);
        ds_val[4] = r4 * dyz;
        ds_val[5] = r4 * dxz;
        ds_val[6] = r4 * dxy;
        ds_val[7] = R(0);
    } else {
        R mxx = 0, myy = 0, mxy = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int ex = S::e(q, 0), ey = S::e(q, 1);
            if (ex) mxx += f[q];
            if (ey) myy += f[q];
            if (ex * ey == 1) mxy += f[q]; else if (ex * ey == -1) mxy -= f[q];
        }
        const R dxx = mxx * inv_rho - (third + u[0] * u[0]);
        const R dyy = myy * inv_rho - (third + u[1] * u[1]);
        const R dxy = mxy * inv_rho - u[0] * u[1];
        const R dT = dxx + dyy, dN = dxx - dyy;
        ds_val[0] = rho * -dT;
        ds_val[1] = R(0.5) * rho * (R(0.5) * (dT + dN));  // x axis
        ds_val[2] = R(0.5) * rho * (R(0.5) * (dT - dN));  // y axis
        ds_val[3] = R(0.25) * rho * dxy;                  // (1,1), (-1,-1)
        ds_val[4] = ds_val[5] = ds_val[6] = ds_val[7] = R(0);
    }
    // delta_s_q: class of q and its sign
    auto ds = [&](int q) -> R {
        if constexpr (S::Q == 27) {
            if (q == 0) return ds_val[0];
            if (q <= 2) return ds_val[1];
            if (q <= 4) return ds_val[2];
            if (q <= 6) return ds_val[3];
            if (q <= 8) return ds_val[4];
            if (q <= 10) return -ds_val[4];
            if (q <= 12) return ds_val[5];
            if (q <= 14) return -ds_val[5];
            if (q <= 16) return ds_val[6];
            if (q <= 18) return -ds_val[6];
            return R(0);
        } else {
            if (q == 0) return ds_val[0];
            if (q == 1 || q == 3) return ds_val[1];
            if (q == 2 || q == 4) return ds_val[2];
            if (q == 5 || q == 7) return ds_val[3];
            return -ds_val[3];
        }
    };
    R dh[S::Q];
    R sum_s = R(0), sum_h = R(0);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        const R feq = feq_q<S>(q, rho, u, uu);
        const R d_s = ds(q);
        dh[q] = f[q] - feq - d_s;
        const R ifeq = kbc_rcp(feq);
        sum_s += d_s * dh[q] * ifeq;
        sum_h += dh[q] * dh[q] * ifeq;
    }
    const R beta = R(cp.beta);
    const R ib = R(1) / beta;
    R gamma = ib - (R(2) - ib) * sum_s / sum_h;
    // kbc_collision.py:155-158: gamma < 1e-15 or NaN -> 2
    if (!(gamma >= R(1e-15))) gamma = R(2);
    const R b2 = R(2) * beta, bg = beta * gamma;
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = f[q] - b2 * ds(q) - bg * dh[q];
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
