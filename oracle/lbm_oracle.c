/* CPU oracle for the lattice Boltzmann step -- TEST INFRASTRUCTURE ONLY.
 * Instantiates lbm_oracle_impl.h for double and float; see lbm_oracle.h. */
#include "lbm_oracle.h"
#include "lbm_oracle_stencils.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define REAL double
#define SFX(name) name##_f64
#include "lbm_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX(name) name##_f32
#include "lbm_oracle_impl.h"
#undef REAL
#undef SFX

int orc_stencil_dq(int stencil, int *d, int *q)
{
    const orc_stencil *st = orc_get_stencil(stencil);
    if (!st) return -1;
    *d = st->d;
    *q = st->q;
    return 0;
}

int orc_run_f64(const orc_problem *p, double *f, double *work, int nsteps, int nthreads)
{ return orc_run_impl_f64(p, f, work, nsteps, nthreads); }
int orc_run_f32(const orc_problem *p, float *f, float *work, int nsteps, int nthreads)
{ return orc_run_impl_f32(p, f, work, nsteps, nthreads); }
int orc_moments_f64(int stencil, const int32_t *res, const double *f, double *rho, double *u, int nthreads)
{ return orc_moments_impl_f64(stencil, res, f, rho, u, nthreads); }
int orc_moments_f32(int stencil, const int32_t *res, const float *f, float *rho, float *u, int nthreads)
{ return orc_moments_impl_f32(stencil, res, f, rho, u, nthreads); }

/* feq of given moment fields: lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24 */
int orc_equilibrium_f64(int stencil, const int32_t *res, const double *rho, const double *u, double *feq, int nthreads)
{
    geom_f64 g;
    if (make_geom_f64(stencil, res, &g)) return -1;
    if (nthreads < 1) nthreads = 1;
    const int64_t N = g.N;
    #pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
        double uu[3], out[27];
        for (int d = 0; d < g.d; ++d) uu[d] = u[(int64_t)d * N + n];
        cell_feq_f64(&g, rho[n], uu, out);
        for (int q = 0; q < g.q; ++q) feq[(int64_t)q * N + n] = out[q];
    }
    return 0;
}
