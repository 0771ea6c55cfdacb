/* Body of the CPU oracle, included once per floating type.
 * Expects REAL (double|float) and SFX(name) to be defined by the includer.
 * TEST INFRASTRUCTURE ONLY -- see lbm_oracle.h for the lettuce citations. */

typedef struct {
    const orc_stencil *st;
    int d, q;
    int64_t X, Y, Z, N;      /* internal 3-D view, Z contiguous */
    int ix[27], iy[27], iz[27]; /* velocities in the internal view */
    int32_t res[3];
    int64_t lstride[3];
    /* the KBC moment tensor e_x^a e_y^b e_z^c of every velocity
     * (kbc_collision.py:22-39), [a*9 + b*3 + c][q] in 3-D, [a*3 + b][q] in
     * 2-D; integer powers of -1, 0, 1, exact in floating point */
    REAL kbc_m[27][27];
} SFX(geom);

static int SFX(make_geom)(int stencil, const int32_t *res, SFX(geom) *g)
{
    const orc_stencil *st = orc_get_stencil(stencil);
    if (!st) return -1;
    g->st = st; g->d = st->d; g->q = st->q;
    int64_t r[3] = {1, 1, 1};
    for (int i = 0; i < st->d; ++i) { if (res[i] <= 0) return -2; r[3 - st->d + i] = res[i]; g->res[i] = res[i]; }
    g->X = r[0]; g->Y = r[1]; g->Z = r[2]; g->N = r[0] * r[1] * r[2];
    for (int qi = 0; qi < st->q; ++qi) {
        int e3[3] = {0, 0, 0};
        for (int i = 0; i < st->d; ++i) e3[3 - st->d + i] = st->e[qi][i];
        g->ix[qi] = e3[0]; g->iy[qi] = e3[1]; g->iz[qi] = e3[2];
    }
    int64_t s = 1;
    for (int i = st->d - 1; i >= 0; --i) { g->lstride[i] = s; s *= res[i]; }
    for (int k = 0; k < 27; ++k)
        for (int qi = 0; qi < 27; ++qi) g->kbc_m[k][qi] = 0;
    if (st->d == 3 && st->q == 27) {
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) for (int c = 0; c < 3; ++c)
            for (int qi = 0; qi < 27; ++qi)
                g->kbc_m[a * 9 + b * 3 + c][qi] = (REAL)(pow((REAL)st->e[qi][0], a) *
                                                         pow((REAL)st->e[qi][1], b) *
                                                         pow((REAL)st->e[qi][2], c));
    } else if (st->d == 2 && st->q == 9) {
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b)
            for (int qi = 0; qi < 9; ++qi)
                g->kbc_m[a * 3 + b][qi] = (REAL)(pow((REAL)st->e[qi][0], a) *
                                                 pow((REAL)st->e[qi][1], b));
    }
    return 0;
}

/* lattice sound speed as lettuce evaluates it: Stencil.cs = 1/sqrt(3) */
static double SFX(cs)(void) { return 1.0 / sqrt(3.0); }

/* lettuce/_flow.py:157-193 (rho = sum_q f, u = (sum_q e f) / rho) */
static void SFX(cell_moments)(const SFX(geom) *g, const REAL *fc, REAL *rho, REAL *u)
{
    REAL r = 0;
    for (int q = 0; q < g->q; ++q) r += fc[q];
    for (int d = 0; d < g->d; ++d) {
        REAL j = 0;
        for (int q = 0; q < g->q; ++q) j += (REAL)g->st->e[q][d] * fc[q];
        u[d] = j / r;
    }
    *rho = r;
}

/* lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24 */
static void SFX(cell_feq)(const SFX(geom) *g, REAL rho, const REAL *u, REAL *feq)
{
    const double cs = SFX(cs)();
    const REAL cs2 = (REAL)(cs * cs);
    REAL uxu = 0;
    for (int d = 0; d < g->d; ++d) uxu += u[d] * u[d];
    for (int q = 0; q < g->q; ++q) {
        REAL exu = 0;
        for (int d = 0; d < g->d; ++d) exu += (REAL)g->st->e[q][d] * u[d];
        REAL a = exu / cs2;
        feq[q] = (REAL)g->st->w[q] * (rho * ((2 * exu - uxu) / (2 * cs2) + (REAL)0.5 * a * a + 1));
    }
}

/* lettuce/ext/_collision/kbc_collision.py:22-39 (moment transform) and
 * :44-94 (shear part s from moments) */
static void SFX(kbc_s)(const SFX(geom) *g, const REAL *fc, REAL *s)
{
    for (int q = 0; q < g->q; ++q) s[q] = 0;
    if (g->d == 3) {
        REAL m[3][3][3];
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) for (int c = 0; c < 3; ++c) {
            REAL acc = 0;
            const REAL *mrow = g->kbc_m[a * 9 + b * 3 + c];
            for (int q = 0; q < 27; ++q) acc += mrow[q] * fc[q];
            m[a][b][c] = acc;
        }
        REAL rho = m[0][0][0];
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) for (int c = 0; c < 3; ++c) m[a][b][c] /= rho;
        m[0][0][0] = rho;
        REAL T = m[2][0][0] + m[0][2][0] + m[0][0][2];
        REAL Nxz = m[2][0][0] - m[0][0][2];
        REAL Nyz = m[0][2][0] - m[0][0][2];
        REAL Pxy = m[1][1][0], Pxz = m[1][0][1], Pyz = m[0][1][1];
        REAL r = m[0][0][0];
        s[0] = r * -T;
        s[1] = (REAL)(1. / 6.) * r * (2 * Nxz - Nyz + T); s[2] = s[1];
        s[3] = (REAL)(1. / 6.) * r * (2 * Nyz - Nxz + T); s[4] = s[3];
        s[5] = (REAL)(1. / 6.) * r * (-Nxz - Nyz + T); s[6] = s[5];
        s[7] = (REAL)(1. / 4) * r * Pyz; s[8] = s[7];
        s[9] = -(REAL)(1. / 4) * r * Pyz; s[10] = s[9];
        s[11] = (REAL)(1. / 4) * r * Pxz; s[12] = s[11];
        s[13] = -(REAL)(1. / 4) * r * Pxz; s[14] = s[13];
        s[15] = (REAL)(1. / 4) * r * Pxy; s[16] = s[15];
        s[17] = -(REAL)(1. / 4) * r * Pxy; s[18] = s[17];
    } else {
        REAL m[3][3];
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
            REAL acc = 0;
            const REAL *mrow = g->kbc_m[a * 3 + b];
            for (int q = 0; q < 9; ++q) acc += mrow[q] * fc[q];
            m[a][b] = acc;
        }
        REAL rho = m[0][0];
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) m[a][b] /= rho;
        m[0][0] = rho;
        REAL T = m[2][0] + m[0][2];
        REAL Nn = m[2][0] - m[0][2];
        REAL Pxy = m[1][1];
        REAL r = m[0][0];
        s[0] = r * -T;
        s[1] = (REAL)0.5 * r * ((REAL)0.5 * (T + Nn));
        s[2] = (REAL)0.5 * r * ((REAL)0.5 * (T - Nn));
        s[3] = (REAL)0.5 * r * ((REAL)0.5 * (T + Nn));
        s[4] = (REAL)0.5 * r * ((REAL)0.5 * (T - Nn));
        s[5] = (REAL)0.25 * r * Pxy;
        s[6] = -s[5];
        s[7] = (REAL)0.25 * r * Pxy;
        s[8] = -s[7];
    }
}

/* u + Force.u_eq: guo.py:30-34 (scale 1/2), shan_chen.py:19-22 (scale tau) */
static void SFX(force_velocity)(const SFX(geom) *g, const orc_problem *p, REAL rho, REAL *u)
{
    if (p->force == ORC_FORCE_NONE) return;
    const REAL scale = p->force == ORC_FORCE_GUO ? (REAL)0.5 : (REAL)(p->force_tau * 1);
    for (int d = 0; d < g->d; ++d) u[d] = u[d] + scale * (REAL)p->accel[d] / rho;
}

/* Guo's source term, guo.py:17-28:
 * (1 - 1/(2 tau)) w_q [(e_q - u)/cs^2 + (e_q.u) e_q/cs^4] . a */
static void SFX(guo_source)(const SFX(geom) *g, const orc_problem *p, const REAL *u, REAL *si)
{
    const double cs = SFX(cs)();
    const REAL cs2 = (REAL)(cs * cs), cs4 = (REAL)(pow(cs, 4));
    for (int q = 0; q < g->q; ++q) {
        REAL eu = 0;
        for (int d = 0; d < g->d; ++d) eu += (REAL)g->st->e[q][d] * u[d];
        REAL acc = 0;
        for (int d = 0; d < g->d; ++d) {
            const REAL e = (REAL)g->st->e[q][d];
            acc += ((e - u[d]) / cs2 + e * eu / cs4) * (REAL)p->accel[d];
        }
        si[q] = (REAL)(1 - 1 / (2 * p->force_tau)) * ((REAL)g->st->w[q] * acc);
    }
}

/* Pi_ab = sum_q e_qa e_qb g_q (lettuce/_flow.py:228-234) */
static void SFX(shear_tensor)(const SFX(geom) *g, const REAL *gq, REAL pi[3][3])
{
    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) pi[a][b] = 0;
    for (int a = 0; a < g->d; ++a) for (int b = 0; b < g->d; ++b) {
        REAL acc = 0;
        for (int q = 0; q < g->q; ++q)
            acc += gq[q] * (REAL)(g->st->e[q][a] * g->st->e[q][b]);
        pi[a][b] = acc;
    }
}

/* one collision at one cell, in place on fc[Q] */
static void SFX(cell_collide)(const SFX(geom) *g, const orc_problem *p, REAL *fc)
{
    const int Q = g->q;
    REAL rho, u[3], feq[27];
    switch (p->collision) {
    case ORC_NO_COLLISION: /* lettuce/ext/_collision/no_collision.py:10-11 */
        return;
    case ORC_BGK: { /* lettuce/ext/_collision/bgk_collision.py:17-22 */
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(force_velocity)(g, p, rho, u);
        SFX(cell_feq)(g, rho, u, feq);
        const REAL omega = (REAL)(1.0 / p->tau);
        REAL si[27] = {0};
        if (p->force == ORC_FORCE_GUO) SFX(guo_source)(g, p, u, si);
        for (int q = 0; q < Q; ++q) fc[q] = fc[q] - omega * (fc[q] - feq[q]) + si[q];
        return;
    }
    case ORC_REGULARIZED: { /* lettuce/ext/_collision/regularized_collision.py:17-47 */
        const double cs = SFX(cs)();
        const REAL cs2 = (REAL)(cs * cs), cs4 = (REAL)pow(cs, 4);
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(cell_feq)(g, rho, u, feq);
        REAL gq[27] = {0}, pi[3][3];
        for (int q = 0; q < Q; ++q) gq[q] = fc[q] - feq[q];
        SFX(shear_tensor)(g, gq, pi);
        for (int q = 0; q < Q; ++q) {
            REAL acc = 0;
            for (int a = 0; a < g->d; ++a) for (int b = 0; b < g->d; ++b) {
                REAL qm = (REAL)(g->st->e[q][a] * g->st->e[q][b]);
                if (a == b) qm -= cs2;
                acc += qm * pi[a][b];
            }
            const REAL fi1 = (REAL)g->st->w[q] * acc / (2 * cs4);
            fc[q] = feq[q] + (1 - (REAL)(1.0 / p->tau)) * fi1;
        }
        return;
    }
    case ORC_MRT: { /* lettuce/ext/_collision/mrt_collision.py:23-30 */
        const double *M = p->mrt_tables, *Mi = M + Q * Q, *sr = Mi + Q * Q;
        REAL m[27], meq[27];
        for (int i = 0; i < Q; ++i) {
            REAL acc = 0;
            for (int q = 0; q < Q; ++q) acc += (REAL)M[i * Q + q] * fc[q];
            m[i] = acc;
            meq[i] = 0;
        }
        const REAL rho = m[0];
        if (p->mrt_equilibrium == ORC_MRT_EQ_DELLAR) {
            const REAL jx = m[1], jy = m[2];
            meq[0] = rho; meq[1] = jx; meq[2] = jy;
            meq[3] = jx * jx / rho * 9 / 2;
            meq[4] = jx * jy / rho * 9;
            meq[5] = jy * jy / rho * 9 / 2;
        } else if (p->mrt_equilibrium == ORC_MRT_EQ_LALLEMAND) {
            const REAL jx = m[1], jy = m[2];
            const REAL c1 = -2, alpha2 = -8, alpha3 = 4, gamma1 = (REAL)(2.0 / 3.0), gamma2 = 18,
                       gamma3 = (REAL)(2.0 / 3.0), gamma4 = -18;
            meq[0] = rho; meq[1] = jx; meq[2] = jy;
            meq[3] = (REAL)0.5 * gamma1 * (jx * jx - jy * jy);
            meq[4] = (REAL)0.5 * gamma3 * (jx * jy);
            meq[5] = (REAL)0.25 * alpha2 * rho + (REAL)(1.0 / 6.0) * gamma2 * (jx * jx + jy * jy);
            meq[6] = (REAL)0.5 * c1 * jx;
            meq[7] = (REAL)0.5 * c1 * jy;
            meq[8] = (REAL)0.25 * alpha3 * rho + (REAL)(1.0 / 6.0) * gamma4 * (jx * jx + jy * jy);
        } else if (p->mrt_equilibrium == ORC_MRT_EQ_HERMITE) {
            const REAL jx = m[1], jy = m[2], jz = m[3];
            const REAL r2 = rho * rho, r3 = r2 * rho, r4 = r3 * rho, r5 = r4 * rho;
            meq[0] = rho; meq[1] = jx; meq[2] = jy; meq[3] = jz;
            meq[4] = jx * jx / rho; meq[5] = jx * jy / rho; meq[6] = jx * jz / rho;
            meq[7] = jy * jy / rho; meq[8] = jy * jz / rho; meq[9] = jz * jz / rho;
            meq[10] = jx * jx * jy / r2; meq[11] = jx * jx * jz / r2; meq[12] = jx * jy * jy / r2;
            meq[13] = jx * jy * jz / r2; meq[14] = jx * jz * jz / r2; meq[15] = jy * jy * jz / r2;
            meq[16] = jy * jz * jz / r2;
            meq[17] = jx * jx * jy * jy / r3; meq[18] = jx * jx * jy * jz / r3;
            meq[19] = jx * jx * jz * jz / r3; meq[20] = jx * jy * jy * jz / r3;
            meq[21] = jx * jy * jz * jz / r3; meq[22] = jy * jy * jz * jz / r3;
            meq[23] = jx * jx * jy * jy * jz / r4; meq[24] = jx * jx * jy * jz * jz / r4;
            meq[25] = jx * jy * jy * jz * jz / r4;
            meq[26] = jx * jy * jx * jz * jy * jz / r5;
        } else { /* the moments of feq(rho, u) (Transform.equilibrium's intent) */
            REAL r0, u0[3];
            SFX(cell_moments)(g, fc, &r0, u0);
            SFX(cell_feq)(g, r0, u0, feq);
            for (int i = 0; i < Q; ++i) {
                REAL acc = 0;
                for (int q = 0; q < Q; ++q) acc += (REAL)M[i * Q + q] * feq[q];
                meq[i] = acc;
            }
        }
        for (int i = 0; i < Q; ++i) m[i] = m[i] - (REAL)(1.0 / sr[i]) * (m[i] - meq[i]);
        for (int q = 0; q < Q; ++q) {
            REAL acc = 0;
            for (int i = 0; i < Q; ++i) acc += (REAL)Mi[q * Q + i] * m[i];
            fc[q] = acc;
        }
        return;
    }
    case ORC_SMAGORINSKY: { /* lettuce/ext/_collision/smagorinsky_collision.py:22-41 */
        const double cs = SFX(cs)();
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(force_velocity)(g, p, rho, u);
        SFX(cell_feq)(g, rho, u, feq);
        REAL gq[27] = {0}, pi[3][3];
        for (int q = 0; q < Q; ++q) gq[q] = fc[q] - feq[q];
        SFX(shear_tensor)(g, gq, pi);
        for (int a = 0; a < g->d; ++a) for (int b = 0; b < g->d; ++b)
            pi[a][b] /= (REAL)(2.0 * rho * (cs * cs));
        REAL tau_eff = (REAL)p->tau;
        const REAL nu = ((REAL)p->tau - (REAL)0.5) / (REAL)3.0;
        for (int it = 0; it < 2; ++it) {
            REAL ss = 0;
            for (int a = 0; a < g->d; ++a) for (int b = 0; b < g->d; ++b) {
                const REAL sab = pi[a][b] / tau_eff;
                ss += sab * sab;
            }
            const REAL nu_t = (REAL)(p->smagorinsky_constant * p->smagorinsky_constant) * ss;
            tau_eff = (nu + nu_t) * (REAL)3.0 + (REAL)0.5;
        }
        REAL si[27] = {0};
        if (p->force == ORC_FORCE_GUO) SFX(guo_source)(g, p, u, si);
        for (int q = 0; q < Q; ++q) fc[q] = fc[q] - (REAL)1.0 / tau_eff * (fc[q] - feq[q]) + si[q];
        return;
    }
    case ORC_TRT: { /* lettuce/ext/_collision/trt_collision.py:16-27 */
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(cell_feq)(g, rho, u, feq);
        REAL out[27];
        const REAL tp2 = (REAL)(2.0 * p->tau), tm2 = (REAL)(2.0 * p->tau_minus);
        for (int q = 0; q < Q; ++q) {
            const int o = g->st->opp[q];
            REAL d = ((fc[q] + fc[o]) - (feq[q] + feq[o])) / tp2;
            d += ((fc[q] - fc[o]) - (feq[q] - feq[o])) / tm2;
            out[q] = fc[q] - d;
        }
        for (int q = 0; q < Q; ++q) fc[q] = out[q];
        return;
    }
    case ORC_KBC: { /* lettuce/ext/_collision/kbc_collision.py:96-160 */
        const REAL beta = (REAL)(1.0 / (2.0 * p->tau));
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(cell_feq)(g, rho, u, feq);
        REAL s1[27], s2[27], ds[27], dh[27];
        SFX(kbc_s)(g, fc, s1);
        SFX(kbc_s)(g, feq, s2);
        REAL sum_s = 0, sum_h = 0;
        for (int q = 0; q < Q; ++q) {
            ds[q] = s1[q] - s2[q];
            dh[q] = fc[q] - feq[q] - ds[q];
        }
        for (int q = 0; q < Q; ++q) sum_s += ds[q] * dh[q] / feq[q];
        for (int q = 0; q < Q; ++q) sum_h += dh[q] * dh[q] / feq[q];
        REAL ib = (REAL)1 / beta;
        REAL gamma = ib - (2 - ib) * sum_s / sum_h;
        if (gamma < (REAL)1e-15) gamma = 2;
        if (gamma != gamma) gamma = 2;
        for (int q = 0; q < Q; ++q) fc[q] = fc[q] - beta * (2 * ds[q] + gamma * dh[q]);
        return;
    }
    }
}

static void SFX(cell_coords)(const SFX(geom) *g, int64_t n, int64_t *c)
{
    for (int i = 0; i < g->d; ++i) c[i] = (n / g->lstride[i]) % g->res[i];
}

/* stream: lettuce/_simulation.py:241-256; f_out[q](x) = f[q](x - e_q) periodic,
 * with the destination keeping its value where no_streaming_mask == 1 */
static void SFX(stream)(const SFX(geom) *g, const orc_problem *p, const REAL *f, REAL *out, int nthreads)
{
    const int64_t X = g->X, Y = g->Y, Z = g->Z, N = g->N;
    for (int q = 0; q < g->q; ++q) {
        const int ex = g->ix[q], ey = g->iy[q], ez = g->iz[q];
        const REAL *src = f + (int64_t)q * N;
        REAL *dst = out + (int64_t)q * N;
        const uint8_t *nsm = p->nsm ? p->nsm + (int64_t)q * N : 0;
        #pragma omp parallel for collapse(2) num_threads(nthreads) schedule(static)
        for (int64_t x = 0; x < X; ++x) {
            for (int64_t y = 0; y < Y; ++y) {
                int64_t xs = (x - ex + X) % X, ys = (y - ey + Y) % Y;
                const REAL *srow = src + (xs * Y + ys) * Z;
                REAL *drow = dst + (x * Y + y) * Z;
                const REAL *own = src + (x * Y + y) * Z;
                if (q == 0) { for (int64_t z = 0; z < Z; ++z) drow[z] = own[z]; continue; }
                for (int64_t z = 0; z < Z; ++z) {
                    int64_t zs = z - ez; zs = zs < 0 ? zs + Z : (zs >= Z ? zs - Z : zs);
                    drow[z] = srow[zs];
                }
                if (nsm) {
                    const uint8_t *mrow = nsm + (x * Y + y) * Z;
                    for (int64_t z = 0; z < Z; ++z) if (mrow[z] == 1) drow[z] = own[z];
                }
            }
        }
    }
}

static int64_t SFX(bcast_index)(const SFX(geom) *g, const int64_t *c, const int64_t *stride)
{
    int64_t k = 0;
    for (int i = 0; i < g->d; ++i) k += c[i] * stride[i];
    return k;
}

/* anti-bounce-back outlet, lettuce/ext/_boundary/anti_bounce_back_outlet.py:71-91:
 * in place on the plane, regardless of the no-collision mask */
static void SFX(anti_bounce_back)(const SFX(geom) *g, const orc_substep *sb, REAL *f)
{
    const int D = g->d, Q = g->q, ax = sb->axis;
    const int64_t n_ax = g->res[ax];
    const int64_t plane = sb->sign > 0 ? n_ax - 1 : 0;
    const int64_t nb = sb->sign > 0 ? n_ax - 2 : 1;
    const double cs = SFX(cs)();
    const REAL cs_r = (REAL)cs, cs4 = (REAL)(cs * cs * cs * cs);
    int vel[27], nv = 0;
    for (int q = 0; q < Q; ++q) {
        int dot = g->st->e[q][ax] * sb->sign;
        if (dot > 1 - 1e-6) vel[nv++] = q;
    }
    const int64_t N = g->N;
    for (int64_t n = 0; n < N; ++n) {
        int64_t c[3];
        SFX(cell_coords)(g, n, c);
        if (c[ax] != plane) continue;
        int64_t cn[3] = {c[0], c[1], c[2]};
        cn[ax] = nb;
        int64_t m = 0;
        for (int i = 0; i < D; ++i) m += cn[i] * g->lstride[i];
        REAL fc[27], fn[27], rho, u[3], rho_n, un[3];
        for (int q = 0; q < Q; ++q) { fc[q] = f[(int64_t)q * N + n]; fn[q] = f[(int64_t)q * N + m]; }
        SFX(cell_moments)(g, fc, &rho, u);
        SFX(cell_moments)(g, fn, &rho_n, un);
        REAL uw[3], uu = 0;
        for (int d = 0; d < D; ++d) { uw[d] = u[d] + (REAL)0.5 * (u[d] - un[d]); uu += uw[d] * uw[d]; }
        REAL nrm = (REAL)sqrt((double)uu) / cs_r;
        for (int k = 0; k < nv; ++k) {
            int v = vel[k];
            REAL eu = 0;
            for (int d = 0; d < D; ++d) eu += (REAL)g->st->e[v][d] * uw[d];
            f[(int64_t)g->st->opp[v] * N + n] =
                -fc[v] + (REAL)g->st->w[v] * rho * (2 + eu * eu / cs4 - nrm * nrm);
        }
    }
}

/* pressure outlet, lettuce/ext/_boundary/equilibrium_outlet_p.py:61-71: in
 * place on the plane, feq(rho_outlet, u of the neighbour plane) */
static void SFX(equilibrium_outlet_p)(const SFX(geom) *g, const orc_substep *sb, REAL *f)
{
    const int D = g->d, Q = g->q, ax = sb->axis;
    const int64_t n_ax = g->res[ax];
    const int64_t plane = sb->sign > 0 ? n_ax - 1 : 0;
    const int64_t nb = sb->sign > 0 ? n_ax - 2 : 1;
    const int64_t N = g->N;
    const REAL rho_w = (REAL)sb->param[0];
    for (int64_t n = 0; n < N; ++n) {
        int64_t c[3] = {0, 0, 0};
        SFX(cell_coords)(g, n, c);
        if (c[ax] != plane) continue;
        int64_t cn[3] = {c[0], c[1], c[2]};
        cn[ax] = nb;
        int64_t m = 0;
        for (int i = 0; i < D; ++i) m += cn[i] * g->lstride[i];
        REAL fn[27], rn, un[3], feq[27];
        for (int q = 0; q < Q; ++q) fn[q] = f[(int64_t)q * N + m];
        SFX(cell_moments)(g, fn, &rn, un);
        SFX(cell_feq)(g, rho_w, un, feq);
        for (int q = 0; q < Q; ++q) f[(int64_t)q * N + n] = feq[q];
    }
}

/* partially saturated cell, lettuce/ext/_boundary/partially_saturated_boundary.py:24-41 */
static void SFX(partially_saturated)(const SFX(geom) *g, const orc_substep *sb, const REAL *fc,
                                     REAL *out)
{
    const int Q = g->q;
    REAL rho, u[3], feq[27], zero[3] = {0, 0, 0}, feq0[27];
    SFX(cell_moments)(g, fc, &rho, u);
    SFX(cell_feq)(g, rho, u, feq);
    SFX(cell_feq)(g, rho, zero, feq0);
    const REAL tau = (REAL)sb->param[0], B = (REAL)sb->param[1];
    for (int q = 0; q < Q; ++q) {
        const int o = g->st->opp[q];
        out[q] = fc[q] - (1 - B) / tau * (fc[q] - feq[q]) + B * ((fc[o] - feq[o]) - (fc[q] - feq0[q]));
    }
}

/* masked collide: lettuce/_simulation.py:258-305 */
static void SFX(collide)(const SFX(geom) *g, const orc_problem *p, REAL *f, int nthreads)
{
    const int Q = g->q;
    const int64_t N = g->N;
    if (!p->ncm) {
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int64_t n = 0; n < N; ++n) {
            REAL fc[27];
            for (int q = 0; q < Q; ++q) fc[q] = f[(int64_t)q * N + n];
            SFX(cell_collide)(g, p, fc);
            for (int q = 0; q < Q; ++q) f[(int64_t)q * N + n] = fc[q];
        }
        return;
    }
    for (int k = 0; k < p->n_sub; ++k) {
        const orc_substep *sb = &p->sub[k];
        if (sb->kind == ORC_SUB_ANTI_BOUNCE_BACK) { SFX(anti_bounce_back)(g, sb, f); continue; }
        if (sb->kind == ORC_SUB_EQUILIBRIUM_OUTLET_P) { SFX(equilibrium_outlet_p)(g, sb, f); continue; }
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int64_t n = 0; n < N; ++n) {
            if (p->ncm[n] != k) continue;
            REAL fc[27], out[27];
            for (int q = 0; q < Q; ++q) fc[q] = f[(int64_t)q * N + n];
            switch (sb->kind) {
            case ORC_SUB_COLLISION: SFX(cell_collide)(g, p, fc); for (int q = 0; q < Q; ++q) out[q] = fc[q]; break;
            case ORC_SUB_BOUNCE_BACK: for (int q = 0; q < Q; ++q) out[q] = fc[g->st->opp[q]]; break;
            case ORC_SUB_EQUILIBRIUM_PU: {
                int64_t c[3]; SFX(cell_coords)(g, n, c);
                const REAL *rb = (const REAL *)sb->rho, *ub = (const REAL *)sb->u;
                REAL rho = rb[SFX(bcast_index)(g, c, sb->rho_stride)];
                REAL u[3];
                int64_t ui = SFX(bcast_index)(g, c, sb->u_stride + 1);
                for (int d = 0; d < g->d; ++d) u[d] = ub[ui + d * sb->u_stride[0]];
                SFX(cell_feq)(g, rho, u, out);
                break;
            }
            case ORC_SUB_PARTIALLY_SATURATED: SFX(partially_saturated)(g, sb, fc, out); break;
            default: for (int q = 0; q < Q; ++q) out[q] = fc[q]; break;
            }
            for (int q = 0; q < Q; ++q) f[(int64_t)q * N + n] = out[q];
        }
    }
}

static int SFX(orc_run_impl)(const orc_problem *p, REAL *f, REAL *work, int nsteps, int nthreads)
{
    SFX(geom) g;
    if (SFX(make_geom)(p->stencil, p->res, &g)) return -1;
    if (p->collision == ORC_KBC && !(g.q == 27 || g.q == 9)) return -2;
    if (nthreads < 1) nthreads = 1;
    const size_t bytes = (size_t)g.q * (size_t)g.N * sizeof(REAL);
    REAL *cur = f, *nxt = work;
    if (p->n_links > 0) {
        /* halfway bounce-back (examples/advanced_projects/
         * efficient_bounce_back_obstacle/boundary/halfway_bounce_back_boundary.py:
         * __call__ :170-190, calc_force_on_boundary :211-218, store_f_collided
         * :220-242) in the EbbSimulation order (simulation/ebb_simulation.py:72-76,
         * 93-101) */
        /* the interpolated links follow linear_interpolated_bounce_back_boundary.py:
         * store_f_collided :128-153, __call__ :55-96, calc_force_on_boundary :104-126 */
        const int64_t K = p->n_links;
        REAL *fcol = (REAL *)malloc((size_t)K * 3 * sizeof(REAL));
        if (!fcol) return -3;
        REAL *fopp = fcol + K, *val = fcol + 2 * K;
        for (int s = 0; s < nsteps; ++s) {
            SFX(collide)(&g, p, cur, nthreads);
            for (int64_t k = 0; k < K; ++k) {
                const int q = (int)p->links[2 * k];
                fcol[k] = cur[q * g.N + p->links[2 * k + 1]];
                fopp[k] = cur[(int64_t)g.st->opp[q] * g.N + p->links[2 * k + 1]];
            }
            SFX(stream)(&g, p, cur, nxt, nthreads);
            { REAL *t = cur; cur = nxt; nxt = t; }
            for (int64_t k = 0; k < K; ++k) {
                const int q = (int)p->links[2 * k];
                const REAL d = p->link_d ? (REAL)p->link_d[k] : (REAL)-1;
                if (d < (REAL)0) {
                    val[k] = fcol[k];
                } else if (d < (REAL)0.5) {
                    const REAL streamed = cur[q * g.N + p->links[2 * k + 1]];
                    val[k] = (REAL)2 * d * fcol[k] + ((REAL)1 - (REAL)2 * d) * streamed;
                } else {
                    val[k] = ((REAL)1 / ((REAL)2 * d)) * fcol[k] +
                             ((REAL)1 - (REAL)1 / ((REAL)2 * d)) * fopp[k];
                }
            }
            double force[3] = {0.0, 0.0, 0.0};
            for (int64_t k = 0; k < K; ++k) {
                const int q = (int)p->links[2 * k];
                cur[(int64_t)g.st->opp[q] * g.N + p->links[2 * k + 1]] = val[k];
                const int mode = p->link_force ? p->link_force[k] : 1;
                const double gb = mode == 2 ? 2.0 * (double)val[k]
                                            : (double)fcol[k] + (double)val[k];
                if (mode == 0) continue;
                for (int d = 0; d < g.d; ++d) force[d] += gb * g.st->e[q][d];
            }
            if (p->force_out)
                for (int d = 0; d < 3; ++d) p->force_out[3 * s + d] = force[d];
        }
        free(fcol);
        if (cur != f) memcpy(f, cur, bytes);
        return 0;
    }
    for (int s = 0; s < nsteps; ++s) {
        const int pre = (p->strategy & ORC_PRE_STREAMING) != 0;
        const int post = (p->strategy & ORC_POST_STREAMING) != 0;
        if (pre) { SFX(stream)(&g, p, cur, nxt, nthreads); REAL *t = cur; cur = nxt; nxt = t; }
        SFX(collide)(&g, p, cur, nthreads);
        if (post) { SFX(stream)(&g, p, cur, nxt, nthreads); REAL *t = cur; cur = nxt; nxt = t; }
    }
    if (cur != f) memcpy(f, cur, bytes);
    return 0;
}

static int SFX(orc_moments_impl)(int stencil, const int32_t *res, const REAL *f, REAL *rho, REAL *u, int nthreads)
{
    SFX(geom) g;
    if (SFX(make_geom)(stencil, res, &g)) return -1;
    if (nthreads < 1) nthreads = 1;
    const int64_t N = g.N;
    #pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
        REAL fc[27], r, uu[3];
        for (int q = 0; q < g.q; ++q) fc[q] = f[(int64_t)q * N + n];
        SFX(cell_moments)(&g, fc, &r, uu);
        rho[n] = r;
        for (int d = 0; d < g.d; ++d) u[(int64_t)d * N + n] = uu[d];
    }
    return 0;
}
