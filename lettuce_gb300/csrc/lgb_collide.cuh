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
//   forced BGK   lettuce/ext/_collision/bgk_collision.py:17-22 with
//                lettuce/ext/_force/guo.py:17-36, shan_chen.py:13-24
//   regularized  lettuce/ext/_collision/regularized_collision.py:17-47
//   Smagorinsky  lettuce/ext/_collision/smagorinsky_collision.py:22-41
//   MRT          lettuce/ext/_collision/mrt_collision.py:23-30 with the
//                equilibria of lettuce/util/moments.py:92-104, 180-204,
//                240-274, 511-545
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

// collision kinds beyond the ABI's: BGK with a body force (the ABI's BGK
// with a force descriptor) is its own kernel variant
constexpr int LGB_BGK_FORCED = 16;

struct CollideParams {
    double omega;        // 1 / tau (BGK)
    double inv_2tp;      // 1 / (2 tau_plus) (TRT)
    double inv_2tm;      // 1 / (2 tau_minus) (TRT)
    double beta;         // 1 / (2 tau) (KBC)
    // body force (forced BGK, Smagorinsky): constant acceleration a (lattice
    // units), equilibrium velocity u = j / rho + ueq_scale a / rho, source
    // term src_scale w_q [(e_q - u) / cs^2 + (e_q . u) e_q / cs^4] . a
    double accel[3];
    double ueq_scale;    // Guo: 1/2; Shan-Chen: the force's tau; none: 0
    double src_scale;    // Guo: 1 - 1 / (2 tau_force); otherwise 0
    double tau;          // Smagorinsky: the molecular relaxation time
    double smag_c2;      // Smagorinsky constant squared
    // the float32 rates of the shifted-space BGK / TRT (lgb_shifted.cuh),
    // rounded once on the host by set_float_rates: (float) omega,
    // (float) (1 - omega), (float) inv_2tp, (float) inv_2tm. Formed per
    // thread from the doubles above they occupied the float64 pipe a fifth
    // of the 16-bit pull launch.
    float f_omega, f_one_minus_omega, f_inv_2tp, f_inv_2tm;
};

// fill the float32 copies of the rates from the float64 ones
LGB_HD void set_float_rates(CollideParams &cp) {
    cp.f_omega = (float)cp.omega;
    cp.f_one_minus_omega = (float)(1.0 - cp.omega);
    cp.f_inv_2tp = (float)cp.inv_2tp;
    cp.f_inv_2tm = (float)cp.inv_2tm;
}

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
// the KBC collision's other quotients (1 / rho, 1 / beta, the entropic
// ratio): the hardware approximation in float32 (__fdividef, within 2 ulp)
// when LGB_KBC_FAST_DIV is 1, exact division in float64. The correctly
// rounded float32 division keeps a longer instruction sequence whose
// registers made the D3Q27 obstacle kernel spill 52 bytes at its 64-register
// bound; with the approximation it spills none: 26.2k -> 27.5k MLUPS on the
// 512x128x128 obstacle (PRE).
#ifndef LGB_KBC_FAST_DIV
#define LGB_KBC_FAST_DIV 1
#endif
LGB_HD float kbc_div(float a, float b) {
#ifdef __CUDA_ARCH__
    if constexpr (LGB_KBC_FAST_DIV) return __fdividef(a, b);
#endif
    return a / b;
}
LGB_HD double kbc_div(double a, double b) { return a / b; }

// the population index of velocity (x, y, z) of a 3-D stencil
template <class S> LGB_HD constexpr int q_of(int x, int y, int z) {
    for (int q = 0; q < S::Q; ++q)
        if (S::e(q, 0) == x && S::e(q, 1) == y && S::e(q, 2) == z) return q;
    return -1;
}

// Where a collision reads and writes a cell's populations: a register array
// (RegPops), or a column of a block's shared-memory stage (lgb_step.cuh,
// StagePops) read back for every pass instead of being held in registers.
// Both evaluate the same operations in the same order.
template <class R, int Q> struct RegPops {
    R (&f)[Q];
    LGB_HD R get(int q) const { return f[q]; }
    LGB_HD void set(int q, R v) const { f[q] = v; }
};

// D3Q27: density, momentum and the second moments m_ab = sum_q e_qa e_qb f_q
// (packed xx, yy, zz, xy, xz, yz) from partial sums along the nine z-lines
// (about 70 additions instead of about 180 for the ten sums taken one by one)
template <class S, class R, class P>
LGB_HD void moments27_of(const P &f, R &rho, R (&j)[3], R (&m)[6]) {
    static_assert(S::Q == 27, "D3Q27 only");
    R A[3][3], B[3][3], C[3][3];  // per (x, y) line: sum f, sum z f, sum z^2 f
#pragma unroll
    for (int x = -1; x <= 1; ++x) {
#pragma unroll
        for (int y = -1; y <= 1; ++y) {
            const R lo = f.get(q_of<S>(x, y, -1)), mid = f.get(q_of<S>(x, y, 0)),
                    hi = f.get(q_of<S>(x, y, 1));
            C[x + 1][y + 1] = hi + lo;
            B[x + 1][y + 1] = hi - lo;
            A[x + 1][y + 1] = C[x + 1][y + 1] + mid;
        }
    }
    R Ax[3], Bx[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        Ax[x] = A[x][0] + A[x][1] + A[x][2];
        Bx[x] = B[x][0] + B[x][1] + B[x][2];
    }
    const R Ayp = A[0][2] + A[1][2] + A[2][2], Aym = A[0][0] + A[1][0] + A[2][0];
    const R Byp = B[0][2] + B[1][2] + B[2][2], Bym = B[0][0] + B[1][0] + B[2][0];
    rho = Ax[0] + Ax[1] + Ax[2];
    j[0] = Ax[2] - Ax[0];
    j[1] = Ayp - Aym;
    j[2] = Bx[0] + Bx[1] + Bx[2];
    m[0] = Ax[2] + Ax[0];
    m[1] = Ayp + Aym;
    m[2] = (C[0][0] + C[0][1] + C[0][2]) + (C[1][0] + C[1][1] + C[1][2]) +
           (C[2][0] + C[2][1] + C[2][2]);
    m[3] = (A[2][2] - A[2][0]) - (A[0][2] - A[0][0]);
    m[4] = Bx[2] - Bx[0];
    m[5] = Byp - Bym;
}

template <class S, class R>
LGB_HD void moments27(const R (&f)[S::Q], R &rho, R (&j)[3], R (&m)[6]) {
    R(&fm)[S::Q] = const_cast<R(&)[S::Q]>(f);
    moments27_of<S>(RegPops<R, S::Q>{fm}, rho, j, m);
}

// Entropic KBC collision (lettuce/ext/_collision/kbc_collision.py:96-160),
// D3Q27 and D2Q9. The shear part delta_s = s(f) - s(feq) is linear in the
// second moments, s(.) of kbc_collision.py:44-94; for the quadratic
// equilibrium those moments are rho (delta_ab / 3 + u_a u_b) exactly (and
// sum_q feq_q = rho), so delta_s is formed from the deviations
// d_ab = m_ab(f) / rho - (delta_ab / 3 + u_a u_b). Then
//   delta_h = f - feq - delta_s,
//   gamma = 1/beta - (2 - 1/beta) <delta_s delta_h / feq> / <delta_h^2 / feq>
// (2 where that is below 1e-15 or NaN) and f <- f - beta (2 delta_s + gamma delta_h).
template <class S, class R, class P>
LGB_HD void collide_kbc_of(const P &f, const CollideParams &cp, R &rho_out) {
    static_assert(S::Q == 27 || S::Q == 9, "KBC is defined for D3Q27 and D2Q9");
    R rho, u[3];
    R m27[6];
    if constexpr (S::Q == 27) {
        moments27_of<S>(f, rho, u, m27);
        const R inv = kbc_div(R(1), rho);
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] *= inv;
    } else {
        R fr[S::Q];
#pragma unroll
        for (int q = 0; q < S::Q; ++q) fr[q] = f.get(q);
        cell_moments<S>(fr, rho, u);
    }
    const R uu = dot_uu<S>(u);
    const R inv_rho = kbc_div(R(1), rho);
    const R third = R(1.0 / 3.0);
    // delta_s by velocity class (index into ds_val below)
    R ds_val[8];
    if constexpr (S::Q == 27) {
        const R mxx = m27[0], myy = m27[1], mzz = m27[2], mxy = m27[3], mxz = m27[4],
                myz = m27[5];
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
            if (ex) mxx += f.get(q);
            if (ey) myy += f.get(q);
            if (ex * ey == 1) mxy += f.get(q); else if (ex * ey == -1) mxy -= f.get(q);
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
    // The entropic sums and the update run over opposite pairs (q, o): the
    // equilibrium's even part w rho (1 - 1.5 u.u + 4.5 (e.u)^2) is shared,
    // its odd part w rho 3 e.u changes sign, and delta_s is the same for
    // both. delta_h is formed twice (for the sums, then for the update)
    // rather than kept in Q more registers.
    const R c0 = R(1) - R(1.5) * uu;
    auto feq_pair = [&](int q, R &fq, R &fo) {
        R eu = R(0);
#pragma unroll
        for (int d = 0; d < S::D; ++d) {
            const int c = S::e(q, d);
            if (c == 1) eu += u[d];
            else if (c == -1) eu -= u[d];
        }
        const R wr = R(S::w(q)) * rho;
        const R even = wr * (c0 + R(4.5) * eu * eu);
        const R odd = wr * (R(3) * eu);
        fq = even + odd;
        fo = even - odd;
    };
    const R feq0 = R(S::w(0)) * rho * c0;
    R sum_s, sum_h;
    {
        const R d_s = ds(0);
        const R dh = f.get(0) - feq0 - d_s;
        const R ifeq = kbc_rcp(feq0);
        sum_s = d_s * dh * ifeq;
        sum_h = dh * dh * ifeq;
    }
#pragma unroll
    for (int q = 1; q < S::Q; ++q) {
        const int o = S::opp(q);
        if (o < q) continue;
        R fq, fo;
        feq_pair(q, fq, fo);
        const R d_s = ds(q);
        const R hq = f.get(q) - fq - d_s, ho = f.get(o) - fo - d_s;
        const R iq = kbc_rcp(fq), io = kbc_rcp(fo);
        sum_s += d_s * (hq * iq + ho * io);
        sum_h += hq * hq * iq + ho * ho * io;
    }
    const R beta = R(cp.beta);
    const R ib = kbc_div(R(1), beta);
    R gamma = ib - kbc_div((R(2) - ib) * sum_s, sum_h);
    // kbc_collision.py:155-158: gamma < 1e-15 or NaN -> 2
    if (!(gamma >= R(1e-15))) gamma = R(2);
    const R b2 = R(2) * beta, bg = beta * gamma;
    {
        const R d_s = ds(0);
        const R f0 = f.get(0);
        f.set(0, f0 - b2 * d_s - bg * (f0 - feq0 - d_s));
    }
#pragma unroll
    for (int q = 1; q < S::Q; ++q) {
        const int o = S::opp(q);
        if (o < q) continue;
        R fq, fo;
        feq_pair(q, fq, fo);
        const R d_s = ds(q);
        const R gq = f.get(q), go = f.get(o);
        const R hq = gq - fq - d_s, ho = go - fo - d_s;
        f.set(q, gq - b2 * d_s - bg * hq);
        f.set(o, go - b2 * d_s - bg * ho);
    }
    rho_out = rho;
}

template <class S, class R>
LGB_HD void collide_kbc(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    collide_kbc_of<S>(RegPops<R, S::Q>{f}, cp, rho_out);
}

// j / rho + ueq_scale a / rho (forced BGK and Smagorinsky,
// bgk_collision.py:18-19 with Force.u_eq)
template <class S, class R>
LGB_HD void forced_velocity(const R (&f)[S::Q], const CollideParams &cp, R &rho, R (&u)[3]) {
    cell_moments<S>(f, rho, u);
    if (cp.ueq_scale != 0.0) {
        const R s = R(cp.ueq_scale) / rho;
#pragma unroll
        for (int d = 0; d < S::D; ++d) u[d] += s * R(cp.accel[d]);
    }
}

// Guo's source term of population q (guo.py:17-28), zero when src_scale is 0
template <class S, class R>
LGB_HD R guo_source(int q, const CollideParams &cp, const R (&u)[3]) {
    R eu = R(0), ea = R(0), ua = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) {
        const int c = S::e(q, d);
        const R a = R(cp.accel[d]);
        if (c == 1) { eu += u[d]; ea += a; }
        else if (c == -1) { eu -= u[d]; ea -= a; }
        ua += u[d] * a;
    }
    // ((e - u) / cs^2 + (e.u) e / cs^4) . a with cs^2 = 1/3
    const R t = R(3) * (ea - ua) + R(9) * eu * ea;
    return R(cp.src_scale) * R(S::w(q)) * t;
}

template <class S, class R>
LGB_HD void collide_bgk_forced(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    forced_velocity<S>(f, cp, rho, u);
    const R uu = dot_uu<S>(u);
    const R om = R(cp.omega);
    const bool src = cp.src_scale != 0.0;
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        R v = f[q] - om * (f[q] - feq_q<S>(q, rho, u, uu));
        if (src) v += guo_source<S>(q, cp, u);
        f[q] = v;
    }
    rho_out = rho;
}

// second moments sum_q e_qa e_qb g_q of g = f - feq, packed (xx, yy, zz, xy,
// xz, yz) (lettuce/_flow.py:228-234 applied to f - feq)
template <class S, class R>
LGB_HD void noneq_shear(const R (&f)[S::Q], R rho, const R (&u)[3], R uu, R (&pi)[6]) {
#pragma unroll
    for (int k = 0; k < 6; ++k) pi[k] = R(0);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        const R g = f[q] - feq_q<S>(q, rho, u, uu);
        const int ex = S::e(q, 0), ey = S::D > 1 ? S::e(q, 1) : 0,
                  ez = S::D > 2 ? S::e(q, 2) : 0;
        if (ex) pi[0] += g;
        if (ey) pi[1] += g;
        if (ez) pi[2] += g;
        if (ex * ey == 1) pi[3] += g; else if (ex * ey == -1) pi[3] -= g;
        if (ex * ez == 1) pi[4] += g; else if (ex * ez == -1) pi[4] -= g;
        if (ey * ez == 1) pi[5] += g; else if (ey * ez == -1) pi[5] -= g;
    }
}

// regularized: f <- feq + (1 - 1/tau) w_q Q_q : Pi_neq / (2 cs^4), with
// Q_q,ab = e_qa e_qb - cs^2 delta_ab (regularized_collision.py:35-47)
template <class S, class R>
LGB_HD void collide_regularized(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    cell_moments<S>(f, rho, u);
    const R uu = dot_uu<S>(u);
    R pi[6];
    noneq_shear<S>(f, rho, u, uu, pi);
    const R third = R(1.0 / 3.0);
    const R trace = pi[0] + pi[1] + pi[2];
    const R k = (R(1) - R(cp.omega)) * R(4.5);  // (1 - 1/tau) / (2 cs^4)
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        const int ex = S::e(q, 0), ey = S::D > 1 ? S::e(q, 1) : 0,
                  ez = S::D > 2 ? S::e(q, 2) : 0;
        R qp = -third * trace;
        if (ex) qp += pi[0];
        if (ey) qp += pi[1];
        if (ez) qp += pi[2];
        const int xy = ex * ey, xz = ex * ez, yz = ey * ez;
        if (xy) qp += R(2 * xy) * pi[3];
        if (xz) qp += R(2 * xz) * pi[4];
        if (yz) qp += R(2 * yz) * pi[5];
        f[q] = feq_q<S>(q, rho, u, uu) + k * R(S::w(q)) * qp;
    }
    rho_out = rho;
}

// Smagorinsky: BGK with tau_eff from two fixed-point iterations of
// nu_eff = (tau - 1/2) / 3 + C^2 S:S, S = Pi_neq / (2 rho cs^2 tau_eff)
// (smagorinsky_collision.py:22-41), plus the optional force
template <class S, class R>
LGB_HD void collide_smagorinsky(R (&f)[S::Q], const CollideParams &cp, R &rho_out) {
    R rho, u[3];
    forced_velocity<S>(f, cp, rho, u);
    const R uu = dot_uu<S>(u);
    R pi[6];
    noneq_shear<S>(f, rho, u, uu, pi);
    const R scale = R(1.5) / rho;  // 1 / (2 rho cs^2)
    // S:S of the symmetric tensor with the off-diagonal entries counted twice
    R ss = R(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) ss += (pi[k] * scale) * (pi[k] * scale);
#pragma unroll
    for (int k = 3; k < 6; ++k) ss += R(2) * (pi[k] * scale) * (pi[k] * scale);
    const R tau = R(cp.tau);
    const R nu = (tau - R(0.5)) / R(3);
    R tau_eff = tau;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const R nu_eff = nu + R(cp.smag_c2) * ss / (tau_eff * tau_eff);
        tau_eff = nu_eff * R(3) + R(0.5);
    }
    const R om = R(1) / tau_eff;
    const bool src = cp.src_scale != 0.0;
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        R v = f[q] - om * (f[q] - feq_q<S>(q, rho, u, uu));
        if (src) v += guo_source<S>(q, cp, u);
        f[q] = v;
    }
    rho_out = rho;
}

// Per-launch tables of a collision, passed by value as a kernel parameter
// (constant bank: the moment transforms read them as instruction operands).
// Only MRT has any.
struct NoTables {};
template <int Q, class R> struct MrtTables {
    R M[Q * Q];      // moment matrix, row-major
    R Minv[Q * Q];   // its inverse
    R inv_s[Q];      // 1 / relaxation time of each moment
    int32_t eq;      // LGB_MRT_EQ_*
};
template <int COLL, class S, class R> struct TablesOf { using type = NoTables; };
template <class S, class R> struct TablesOf<LGB_MRT, S, R> { using type = MrtTables<S::Q, R>; };

// MRT: m = M f, m <- m - (m - meq) / s, f = M^-1 m
template <class S, class R>
LGB_HD void collide_mrt(R (&f)[S::Q], const MrtTables<S::Q, R> &t, R &rho_out) {
    constexpr int Q = S::Q;
    R m[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        R acc = R(0);
#pragma unroll
        for (int q = 0; q < Q; ++q) acc += t.M[i * Q + q] * f[q];
        m[i] = acc;
    }
    R meq[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) meq[i] = R(0);
    const R rho = m[0];
    if (t.eq == LGB_MRT_EQ_GENERIC) {
        // Transform.equilibrium: the moments of feq(rho, u) of the populations
        R r, u[3];
        cell_moments<S>(f, r, u);
        const R uu = dot_uu<S>(u);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const R e = feq_q<S>(q, r, u, uu);
#pragma unroll
            for (int i = 0; i < Q; ++i) meq[i] += t.M[i * Q + q] * e;
        }
    } else if constexpr (Q == 9) {
        const R jx = m[1], jy = m[2];
        meq[0] = rho; meq[1] = jx; meq[2] = jy;
        if (t.eq == LGB_MRT_EQ_DELLAR) {            // moments.py:180-204
            meq[3] = jx * jx / rho * R(9) / R(2);
            meq[4] = jx * jy / rho * R(9);
            meq[5] = jy * jy / rho * R(9) / R(2);
        } else {                                    // Lallemand & Luo, moments.py:240-274
            const R jj = jx * jx + jy * jy;
            meq[3] = R(1.0 / 2.0 * (2.0 / 3.0)) * (jx * jx - jy * jy);
            meq[4] = R(1.0 / 2.0 * (2.0 / 3.0)) * (jx * jy);
            meq[5] = R(1.0 / 4.0 * -8.0) * rho + R(1.0 / 6.0 * 18.0) * jj;
            meq[6] = R(1.0 / 2.0 * -2.0) * jx;
            meq[7] = R(1.0 / 2.0 * -2.0) * jy;
            meq[8] = R(1.0 / 4.0 * 4.0) * rho + R(1.0 / 6.0 * -18.0) * jj;
        }
    } else if constexpr (Q == 27) {                 // Hermite, moments.py:511-545
        const R jx = m[1], jy = m[2], jz = m[3];
        const R r2 = rho * rho, r3 = r2 * rho, r4 = r3 * rho, r5 = r4 * rho;
        meq[0] = rho; meq[1] = jx; meq[2] = jy; meq[3] = jz;
        meq[4] = jx * jx / rho; meq[5] = jx * jy / rho; meq[6] = jx * jz / rho;
        meq[7] = jy * jy / rho; meq[8] = jy * jz / rho; meq[9] = jz * jz / rho;
        meq[10] = jx * jx * jy / r2; meq[11] = jx * jx * jz / r2;
        meq[12] = jx * jy * jy / r2; meq[13] = jx * jy * jz / r2;
        meq[14] = jx * jz * jz / r2; meq[15] = jy * jy * jz / r2;
        meq[16] = jy * jz * jz / r2;
        meq[17] = jx * jx * jy * jy / r3; meq[18] = jx * jx * jy * jz / r3;
        meq[19] = jx * jx * jz * jz / r3; meq[20] = jx * jy * jy * jz / r3;
        meq[21] = jx * jy * jz * jz / r3; meq[22] = jy * jy * jz * jz / r3;
        meq[23] = jx * jx * jy * jy * jz / r4; meq[24] = jx * jx * jy * jz * jz / r4;
        meq[25] = jx * jy * jy * jz * jz / r4;
        meq[26] = jx * jy * jx * jz * jy * jz / r5;
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) m[i] = m[i] - t.inv_s[i] * (m[i] - meq[i]);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        R acc = R(0);
#pragma unroll
        for (int i = 0; i < Q; ++i) acc += t.Minv[q * Q + i] * m[i];
        f[q] = acc;
    }
    rho_out = rho;
}

template <int COLL, class S, class R, class TT = NoTables>
LGB_HD void collide(R (&f)[S::Q], const CollideParams &cp, R &rho_out, const TT &tab = TT()) {
    if constexpr (COLL == LGB_BGK) {
        collide_bgk<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_TRT) {
        collide_trt<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_KBC) {
        collide_kbc<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_BGK_FORCED) {
        collide_bgk_forced<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_REGULARIZED) {
        collide_regularized<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_SMAGORINSKY) {
        collide_smagorinsky<S>(f, cp, rho_out);
    } else if constexpr (COLL == LGB_MRT) {
        collide_mrt<S>(f, tab, rho_out);
    } else {
        R r = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) r += f[q];
        rho_out = r;
    }
}

}  // namespace lgb
