/*
 * CPU oracle for the lattice Boltzmann step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of lettuce's torch step (stream by periodic roll,
 * masked collide substeps, boundary operators), used by the test-suite as
 * the reference of its comparisons and by bench.py as the timed CPU
 * baseline. Nothing in the
 * product (lettuce_gb300/) links, loads or calls it.
 *
 * Each routine cites the lettuce source it restates (paths are relative to
 * the lettuce project root):
 *   stream          lettuce/_simulation.py:241-256
 *   masked collide  lettuce/_simulation.py:258-305
 *   strategies      lettuce/_simulation.py:148-166
 *   moments         lettuce/_flow.py:157-193
 *   equilibrium     lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24
 *   BGK             lettuce/ext/_collision/bgk_collision.py:17-22
 *   TRT             lettuce/ext/_collision/trt_collision.py:16-27
 *   KBC             lettuce/ext/_collision/kbc_collision.py:22-160
 *   regularized     lettuce/ext/_collision/regularized_collision.py:17-47
 *   Smagorinsky     lettuce/ext/_collision/smagorinsky_collision.py:22-41
 *   forces          lettuce/ext/_force/guo.py:17-36, shan_chen.py:13-24
 *   MRT             lettuce/ext/_collision/mrt_collision.py:23-30
 *   bounce-back     lettuce/ext/_boundary/bounce_back_boundary.py:17-18
 *   equilibrium BC  lettuce/ext/_boundary/equilibrium_boundary_pu.py:79-84
 *   anti-bounce-back outlet
 *                   lettuce/ext/_boundary/anti_bounce_back_outlet.py:71-91
 *   pressure outlet lettuce/ext/_boundary/equilibrium_outlet_p.py:61-71
 *   partially saturated cells
 *                   lettuce/ext/_boundary/partially_saturated_boundary.py:24-41
 *   halfway bounce-back (lettuce's example project)
 *                   examples/advanced_projects/efficient_bounce_back_obstacle/
 *                   boundary/halfway_bounce_back_boundary.py:170-242 and
 *                   simulation/ebb_simulation.py:72-101
 *   interpolated bounce-back (same project)
 *                   boundary/linear_interpolated_bounce_back_boundary.py:55-153
 *   post-streaming full-way bounce-back (same project)
 *                   boundary/fullway_bounce_back_boundary.py:137-178
 *
 * Parity of this restatement with lettuce itself is pinned by golden
 * vectors generated from lettuce (tests/golden/make_golden.py).
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* stencil ids (same numbering as the CUDA library) */
enum { ORC_D1Q3 = 1, ORC_D2Q9 = 2, ORC_D3Q15 = 3, ORC_D3Q19 = 4, ORC_D3Q27 = 5 };
/* collision kinds */
enum { ORC_NO_COLLISION = 0, ORC_BGK = 1, ORC_TRT = 2, ORC_KBC = 3, ORC_REGULARIZED = 4,
       ORC_SMAGORINSKY = 5, ORC_MRT = 6 };
/* MRT equilibrium moments: lettuce/util/moments.py D2Q9Dellar (:180-204),
 * D2Q9Lallemand (:240-274), D3Q27Hermite (:511-545) */
enum { ORC_MRT_EQ_DELLAR = 1, ORC_MRT_EQ_LALLEMAND = 2, ORC_MRT_EQ_HERMITE = 3 };
/* body forces (BGK and Smagorinsky) */
enum { ORC_FORCE_NONE = 0, ORC_FORCE_GUO = 1, ORC_FORCE_SHAN_CHEN = 2 };
/* substep kinds */
enum { ORC_SUB_COLLISION = 0, ORC_SUB_BOUNCE_BACK = 1, ORC_SUB_EQUILIBRIUM_PU = 2,
       ORC_SUB_ANTI_BOUNCE_BACK = 3, ORC_SUB_NONE = 4, ORC_SUB_EQUILIBRIUM_OUTLET_P = 5,
       ORC_SUB_PARTIALLY_SATURATED = 6 };
/* streaming strategies: lettuce's StreamingStrategy enum values
 * (lettuce/cuda_native/_default_code_gen.py:13-17) */
enum { ORC_NO_STREAMING = 0, ORC_POST_STREAMING = 1, ORC_PRE_STREAMING = 2,
       ORC_DOUBLE_STREAMING = 3 };

typedef struct {
    int32_t kind;
    /* equilibrium BC: density (lattice units) and velocity (lattice units),
     * broadcast over the grid by element strides (0 = broadcast dim).
     * strides are given per lettuce dimension (x, y, z order). */
    const void *rho;
    const void *u;
    int64_t rho_stride[3];
    int64_t u_stride[4]; /* [component, x, y, z] */
    /* outlet planes: lettuce dimension index of the normal and its sign */
    int32_t axis;
    int32_t sign;
    /* pressure outlet: [0] = outlet density; partially saturated: tau, B */
    double param[2];
} orc_substep;

typedef struct {
    int32_t stencil;
    int32_t res[3];          /* lettuce resolution; unused trailing dims = 1 */
    int32_t collision;
    int32_t strategy;
    double tau;
    double tau_minus;
    const uint8_t *ncm;      /* [N] substep index per cell, or NULL */
    const uint8_t *nsm;      /* [Q][N] no-streaming values, or NULL */
    int32_t n_sub;
    int32_t collision_index;
    const orc_substep *sub;  /* [n_sub] */
    int32_t force;           /* ORC_FORCE_* */
    double force_tau;
    double accel[3];         /* lattice units */
    double smagorinsky_constant;
    int32_t mrt_equilibrium;
    const double *mrt_tables; /* M [Q][Q], M^-1 [Q][Q], relaxation times [Q] */
    /* halfway bounce-back links. With n_links > 0 every step runs in the
     * order of the example EbbSimulation (collide, stream, post-streaming
     * boundaries) whatever `strategy` says: link k sets population
     * opp(q_k) of fluid cell n_k, after the stream, to the value that
     * cell's population q_k had after the collision (q_k points from the
     * fluid cell into the solid). The momentum-exchange force of step s,
     * 2 sum_k f*_{q_k}(n_k) e_{q_k}, goes to force_out[3 s .. 3 s + 2]. */
    int64_t n_links;
    const int64_t *links;     /* [n_links][2]: q_k, flat cell index n_k */
    double *force_out;        /* [nsteps][3] or NULL */
    /* linear interpolated bounce-back (Bouzidi): wall distance d_k of each
     * link, < 0 for a halfway link (NULL: all halfway). With g = f*_{q_k}:
     * d < 1/2: 2 d g + (1 - 2 d) f_{q_k}(n_k) (the streamed value),
     * d >= 1/2: g / (2 d) + (1 - 1 / (2 d)) f*_{opp(q_k)}(n_k); all links
     * read the field before any is bounced. The force of a step is
     * sum_k (g_k + bounced_k) e_{q_k} (2 g_k e_{q_k} for a halfway link). */
    const double *link_d;
    /* [n_links] how a link counts in force_out: 0 not, 1 (g + bounced) e_q,
     * 2 2 f_q(n) e_q with f_q(n) the streamed value (the post-streaming
     * full-way bounce-back, whose links sit on solid cells and use
     * d = 0); NULL = all 1 */
    const uint8_t *link_force;
} orc_problem;

int orc_stencil_dq(int stencil, int *d, int *q);

/* nsteps full steps in place on f ([Q][N], lettuce layout); work is a
 * [Q][N] scratch buffer. Returns 0 on success. */
int orc_run_f64(const orc_problem *p, double *f, double *work, int nsteps, int nthreads);
int orc_run_f32(const orc_problem *p, float *f, float *work, int nsteps, int nthreads);

/* density [N] and velocity [D][N] of f */
int orc_moments_f64(int stencil, const int32_t *res, const double *f, double *rho, double *u, int nthreads);
int orc_moments_f32(int stencil, const int32_t *res, const float *f, float *rho, float *u, int nthreads);

/* quadratic equilibrium of rho [N], u [D][N] into feq [Q][N] */
int orc_equilibrium_f64(int stencil, const int32_t *res, const double *rho, const double *u, double *feq, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
