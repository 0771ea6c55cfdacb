/*
 * lettuce_gb300 -- C ABI of the GB300 (sm_103a) lattice Boltzmann step.
 *
 * Plain C: device pointers, sizes and scalars only. Every call is
 * asynchronous on the CUDA stream it is given (a cudaStream_t passed as
 * void*, NULL = legacy default stream); nothing here allocates device memory
 * or synchronises. (lgb_step creates, once per host thread and device and
 * outside stream captures, a second stream and two events: a step with an
 * outlet plane runs the plane's launch on it, forked from and joined back
 * into the given stream.) Errors: a non-zero return code and a message from
 * lgb_last_error(); no call traps or aborts on the device.
 *
 * Layout of a population field: lettuce's [Q, *resolution], C-contiguous,
 * the last lettuce dimension fastest (lettuce/_flow.py:92). The q ordering is
 * lettuce's (the stencil modules in lettuce/ext/_stencil/).
 */
#ifndef LETTUCE_GB300_H
#define LETTUCE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGB_ABI_VERSION 5
#define LGB_MAX_SUBSTEPS 8

/* stencils (lettuce/ext/_stencil/d1q3.py, d2q9.py, d3q15.py, d3q19.py, d3q27.py) */
enum { LGB_D1Q3 = 1, LGB_D2Q9 = 2, LGB_D3Q15 = 3, LGB_D3Q19 = 4, LGB_D3Q27 = 5 };

/* population storage. The *_SHIFTED formats hold f_q - w_q in 16 bits; the
 * collision arithmetic runs in float32 for them and for LGB_F32, in float64
 * for LGB_F64. */
enum { LGB_F64 = 0, LGB_F32 = 1, LGB_F16_SHIFTED = 2, LGB_BF16_SHIFTED = 3 };

/* collision operators (lettuce/ext/_collision/): no_collision.py,
 * bgk_collision.py, trt_collision.py, kbc_collision.py,
 * regularized_collision.py, smagorinsky_collision.py */
enum {
    LGB_NO_COLLISION = 0, LGB_BGK = 1, LGB_TRT = 2, LGB_KBC = 3, LGB_REGULARIZED = 4,
    LGB_SMAGORINSKY = 5, LGB_MRT = 6
};

/* equilibrium moments of the MRT collision (lettuce/ext/_collision/mrt_collision.py
 * with the transforms of lettuce/util/moments.py): GENERIC = M feq(rho, u)
 * (Transform.equilibrium), DELLAR / LALLEMAND = the D2Q9 bases' formulas,
 * HERMITE = the D3Q27 Hermite basis' formulas */
enum { LGB_MRT_EQ_GENERIC = 0, LGB_MRT_EQ_DELLAR = 1, LGB_MRT_EQ_LALLEMAND = 2,
       LGB_MRT_EQ_HERMITE = 3 };

/* body forces of BGK and Smagorinsky (lettuce/ext/_force/guo.py,
 * shan_chen.py): a constant acceleration in lattice units */
enum { LGB_FORCE_NONE = 0, LGB_FORCE_GUO = 1, LGB_FORCE_SHAN_CHEN = 2 };

/* substeps of the masked collide, in lettuce's order pre-boundaries,
 * collision, post-boundaries (lettuce/_simulation.py:258-305) */
enum {
    LGB_SUB_COLLISION = 0,
    LGB_SUB_BOUNCE_BACK = 1,       /* lettuce/ext/_boundary/bounce_back_boundary.py */
    LGB_SUB_EQUILIBRIUM_PU = 2,    /* lettuce/ext/_boundary/equilibrium_boundary_pu.py */
    LGB_SUB_ANTI_BOUNCE_BACK = 3,  /* lettuce/ext/_boundary/anti_bounce_back_outlet.py */
    LGB_SUB_NONE = 4,
    LGB_SUB_EQUILIBRIUM_OUTLET_P = 5, /* lettuce/ext/_boundary/equilibrium_outlet_p.py */
    LGB_SUB_PARTIALLY_SATURATED = 6   /* lettuce/ext/_boundary/partially_saturated_boundary.py */
};
/* At most one outlet-plane substep (anti-bounce-back or pressure outlet)
 * per step descriptor. */

/* memory access pattern of one launch. PULL is stream-then-collide
 * (lettuce PRE_STREAMING), PUSH collide-then-stream (POST_STREAMING), LOCAL
 * collide only (NO_STREAMING), STREAM_ONLY streams without collide. The
 * AA pair runs in place (f_out == f_in): AA_EVEN collides and stores every
 * population into its opposite slot, AA_ODD gathers from the neighbours'
 * opposite slots and scatters to the neighbours; an EVEN+ODD pair equals two
 * PUSH steps. AA_UNPACK copies a field left by AA_EVEN (stream pending) into
 * a second field in natural layout, without collision. */
enum {
    LGB_PULL = 0, LGB_PUSH = 1, LGB_LOCAL = 2, LGB_AA_EVEN = 3, LGB_AA_ODD = 4,
    LGB_STREAM_ONLY = 5, LGB_AA_UNPACK = 6
};

/* per-cell flag byte: low 5 bits = substep index (lettuce's
 * no_collision_mask value); bit 7 = the cell has no-streaming bits; bit 6 =
 * some neighbour x + e_q does not stream population q (read only under
 * LGB_OPT_PUSH_GUARD); bit 5 = the cell has halfway bounce-back links
 * (read only when the descriptor's link_bits is set) */
#define LGB_FLAG_INDEX_MASK 0x1f
#define LGB_FLAG_LINKS 0x20
#define LGB_FLAG_PUSH_GUARD 0x40
#define LGB_FLAG_NO_STREAM 0x80

typedef struct {
    int32_t kind;
    /* anti-bounce-back: lettuce dimension of the outflow normal and its sign */
    int32_t axis;
    int32_t sign;
    int32_t reserved;
    /* equilibrium BC: density and velocity in lattice units, in the compute
     * type (double for LGB_F64, float otherwise), broadcast by element
     * strides per lettuce dimension (0 = broadcast) */
    const void *rho;
    const void *u;
    int64_t rho_stride[3];
    int64_t u_stride[4]; /* component, then lettuce dimensions */
    /* pressure outlet: param[0] = outlet density (lattice units);
     * partially saturated: param[0] = tau, param[1] = B(saturation, tau) */
    double param[2];
} lgb_substep;

typedef struct {
    int32_t abi_version;     /* LGB_ABI_VERSION */
    int32_t stencil;
    int32_t storage;
    int32_t collision;
    int32_t pattern;
    int32_t res[3];          /* lettuce resolution; unused trailing dims = 1 */
    double tau;              /* BGK, KBC, regularized and Smagorinsky tau; TRT tau_plus */
    double tau_minus;        /* TRT */
    const void *f_in;        /* [Q][N] in `storage` */
    void *f_out;             /* [Q][N]; == f_in for LGB_LOCAL / AA patterns */
    const uint8_t *flags;    /* [N] or NULL (no boundaries) */
    const uint32_t *no_stream_bits; /* [N] bit q = population q does not stream */
    int32_t n_sub;
    int32_t collision_index;
    lgb_substep sub[LGB_MAX_SUBSTEPS];
    uint32_t *status;        /* optional device word; bit 0 set on a non-finite density */
    int32_t options;         /* LGB_OPT_* bits */
    int32_t force;           /* LGB_FORCE_*; BGK and Smagorinsky only */
    double force_tau;        /* the force's tau (Guo: source factor 1 - 1/(2 tau);
                                Shan-Chen: velocity shift tau a / rho) */
    double accel[3];         /* acceleration, lattice units, lettuce dimension order */
    double smagorinsky_constant; /* LGB_SMAGORINSKY: C (lettuce default 0.17) */
    int32_t mrt_equilibrium;  /* LGB_MRT: LGB_MRT_EQ_* */
    int32_t reserved2;
    const double *mrt_tables; /* LGB_MRT, HOST memory read during the call: the
                                 moment matrix M [Q][Q] (row-major), its inverse
                                 [Q][Q] and the Q relaxation times s_i
                                 (m_i <- m_i - (m_i - meq_i) / s_i) */
    /* Halfway bounce-back of the post-streaming boundaries of lettuce's
     * example project (examples/advanced_projects/efficient_bounce_back_obstacle/
     * boundary/halfway_bounce_back_boundary.py:170-242, applied after the
     * stream by simulation/ebb_simulation.py:72-101). Patterns that stream
     * by pulling (LGB_PULL, LGB_STREAM_ONLY) read link_bits[n] at the cells
     * whose flags carry LGB_FLAG_LINKS: bit q set = population q is not
     * pulled from x - e_q (a solid cell) but takes the cell's own
     * post-collision population opp(q). NULL = no links. */
    const uint32_t *link_bits;   /* [N] */
    /* Interpolated links, the linear interpolated bounce-back of the same
     * project (boundary/linear_interpolated_bounce_back_boundary.py:55-96).
     * With link_val set, every linked population takes link_val[k],
     * k = link_base[n] + (number of link bits below q in link_bits[n]).
     * LGB_PULL and LGB_STREAM_ONLY launches first fill link_val from f_in
     * for the n_links links: link_pairs holds (q, n), q pointing from cell
     * n into the solid, sorted by n and then by opp(q); link_d the wall
     * distance d (< 0: a halfway link, f*_q(n)); g = f*_q(n):
     *   d < 1/2:  2 d g + (1 - 2 d) f*_q(n - e_q)
     *   d >= 1/2: g / (2 d) + (1 - 1 / (2 d)) f*_{opp(q)}(n).
     * link_val is scratch of n_links elements in the field's storage format
     * (the interpolated value is stored like any population). NULL
     * link_val: every link is a halfway link. */
    const uint32_t *link_base;   /* [N] */
    const uint32_t *link_pairs;  /* [n_links][2] */
    const double *link_d;        /* [n_links] */
    void *link_val;              /* [n_links] */
    int64_t n_links;
    /* Momentum exchange on the links of one boundary
     * (halfway_bounce_back_boundary.py:211-218,
     * linear_interpolated_bounce_back_boundary.py:104-126): force_links
     * holds n_force_links triplets (q, n, k), q pointing from cell n into
     * the solid, k the link's index in link_val or 0xffffffff for a halfway
     * link; k with bit 31 set marks a link of the post-streaming full-way
     * bounce-back (fullway_bounce_back_boundary.py:137-178: a solid-cell
     * link of distance 0, counted as 2 b e_q with b its streamed value,
     * entry k & 0x7fffffff). LGB_PULL and LGB_STREAM_ONLY launches, whose stream crosses the
     * links, write sum (f*_q(n) + b) e_q, b = link_val[k] or f*_q(n)
     * (f* = the post-collision field f_in), to force_out (float64 [3],
     * lattice units, lettuce dimension order; unused trailing entries 0);
     * LGB_LOCAL leaves it. Device memory; NULL / 0 = not computed. */
    const uint32_t *force_links; /* [n_force_links][3] */
    int64_t n_force_links;
    double *force_out;
    /* device scratch for the force's partial sums, float64
     * [3 * ceil(n_force_links / LGB_LINK_FORCE_BLOCK)]; needed with
     * force_out (the blocks' partial sums are added in a fixed order, so
     * the force does not depend on scheduling) */
    double *force_scratch;
} lgb_step_desc;

/* links per block of the momentum-exchange reduction */
#define LGB_LINK_FORCE_BLOCK 256

/* options: run the one-cell-per-thread kernel even where the two-cell
 * kernel of the 16-bit formats applies (results are bit-identical) */
#define LGB_OPT_ONE_CELL 1
/* the flags carry LGB_FLAG_PUSH_GUARD: in the PUSH pattern a cell reads its
 * destinations' no-streaming bits only when its own guard bit is set (without
 * this option every cell reads them for every population) */
#define LGB_OPT_PUSH_GUARD 2

/* ABI version of the loaded library */
int lgb_abi_version(void);
/* message of the last failing call on this host thread ("" if none) */
const char *lgb_last_error(void);

/* One stream+collide step over the whole grid.
 * Replaces the generated binding `cuda_native.lettuce(f, f_next, ncm, nsm,
 * tau_inv, velocity_k, density_k, ...)` of lettuce/cuda_native/_template.py:47-53,
 * 72-81 (body from lettuce/cuda_native/_default_code_gen.py:285-316) and the
 * torch step lettuce/_simulation.py:148-166, 241-305 it reproduces. */
int lgb_step(const lgb_step_desc *desc, void *stream);

/* Density [N] and velocity [D][N] (lattice units) of a population field, in
 * float64 when `storage` is LGB_F64 and float32 otherwise.
 * Replaces lettuce/_flow.py:157-193 (Flow.rho / Flow.j / Flow.u).
 * aa_pending != 0 reads a field left by an LGB_AA_EVEN launch (populations in
 * their opposite slots, stream pending). */
int lgb_moments(int32_t stencil, int32_t storage, const int32_t *res,
                const void *f, int32_t aa_pending, void *rho, void *u,
                void *stream);

/* Float64 reductions of a population field into out[LGB_REDUCE_FIELDS]:
 *   [0] sum of rho over the box,           [1] sum of 0.5*|u|^2 over the box,
 *   [2] max |u|^2 over the box,            [3] cells with a non-finite rho,
 *   [4] sum of rho over box cells where mask != 0 (mask may be NULL).
 * The box is [lo, hi) per lettuce dimension. `scratch` must hold
 * lgb_reduce_scratch_bytes() bytes of device memory.
 * Replaces the per-report reductions of
 * lettuce/ext/_reporter/observable_reporter.py:34-42 (IncompressibleKineticEnergy),
 * :27-31 (MaximumVelocity), :140-158 (Mass) and lettuce/_flow.py:200-204. */
#define LGB_REDUCE_FIELDS 5
int64_t lgb_reduce_scratch_bytes(void);
int lgb_reduce(int32_t stencil, int32_t storage, const int32_t *res,
               const void *f, int32_t aa_pending, const int32_t *lo,
               const int32_t *hi, const uint8_t *mask, double *out,
               void *scratch, void *stream);

/* The same float64 reductions as lgb_reduce, for callers that cannot
 * allocate device memory: for example a host code whose device memory is
 * entirely reserved by another allocator (a framework's caching pool, a
 * fixed arena of a Fortran/C solver), or a latency-critical loop where the
 * implicit device synchronisation of cudaMalloc is not acceptable. No
 * counterpart in lettuce (its reductions are torch calls that allocate).
 *
 * Scratch: a file-scope device array of LGB_REDUCE_STATIC_SCRATCH_BYTES
 * (48,640 bytes), held by every GPU that loads this library until the
 * process exits. The reduction's scratch need does not grow with the field
 * (a fixed grid of 1216 partial sums of 5 doubles, checked against the array
 * size when the library is compiled), so every grid the library accepts
 * fits. The call allocates nothing (no cudaMalloc, no allocating library
 * routine).
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the
 * process; make that first call before any stream capture. The kept address
 * belongs to the device's context of that time: after cudaDeviceReset on a
 * device, do not call lgb_reduce_static on it again in this process (reload
 * is not supported). All calls share the one array: calls that
 * overlap on the GPU (different streams, no ordering between them) race and
 * corrupt each other's results -- order them (same stream or events). The
 * array keeps the last call's partial sums; each call writes every partial
 * it reads, so nothing needs clearing. */
#define LGB_REDUCE_STATIC_SCRATCH_BYTES 48640
int lgb_reduce_static(int32_t stencil, int32_t storage, const int32_t *res,
                      const void *f, int32_t aa_pending, const int32_t *lo,
                      const int32_t *hi, const uint8_t *mask, double *out,
                      void *stream);

/* ---- initial fields and the enstrophy observable ------------------------ */

/* Quadratic equilibrium populations of given density and velocity fields
 * (lattice units, in the compute type: double for LGB_F64 storage, float
 * otherwise), broadcast by element strides per lettuce dimension (0 =
 * broadcast; u_stride[0] is the component stride), written into f ([Q][N]
 * in `storage`) when f is not NULL. With rho_out / u_out (both or neither)
 * the density [N] and velocity [D][N] of that equilibrium -- the moments
 * lettuce reads back from the field it has just set -- are written as well;
 * f may then be NULL. Replaces the initial equilibrium of
 * lettuce/_flow.py:127-143 (Flow.initialize), evaluated in the order of
 * lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24. */
int lgb_equilibrium(int32_t stencil, int32_t storage, const int32_t *res, const void *rho,
                    const int64_t *rho_stride, const void *u, const int64_t *u_stride,
                    void *f, void *rho_out, void *u_out, void *stream);

/* f = feq(rho, u) - fneq with the first-order non-equilibrium part
 * fneq_q = w_q tau rho (d_b u_a) (e_qa e_qb - cs^2 delta_ab) / cs^2, the
 * velocity gradient by 6th-order periodic central differences; rho [N] and
 * u [D][N] contiguous in the compute type, D = 2 or 3. Replaces
 * lettuce/_flow.py:341-367 (initialize_f_neq) with the differences of
 * lettuce/util/utility.py:37-99 (torch_gradient, order 6). */
int lgb_init_fneq(int32_t stencil, int32_t storage, const int32_t *res, const void *rho,
                  const void *u, double tau, void *f, void *stream);

/* out[0] = sum over cells of |curl u|^2 (2-D: (d_1 u_0 - d_0 u_1)^2; 3-D the
 * three components), u [dims][N] contiguous in float64 (precision LGB_F64)
 * or float32 (LGB_F32), lattice units, derivatives by 6th-order periodic
 * central differences with dx = 1, accumulated in float64 through a fixed
 * grid of partial sums folded in a fixed order. `scratch`: device memory of
 * lgb_reduce_scratch_bytes() bytes. Enstrophy in physical units is
 * out[0] * (u_pu / u_lu)^2 * dx^(dims - 2). Replaces
 * lettuce/ext/_reporter/observable_reporter.py:45-67 (Enstrophy). */
int lgb_enstrophy(int32_t dims, int32_t precision, const int32_t *res, const void *u,
                  double *out, void *scratch, void *stream);

/* ---- batched domains ---------------------------------------------------
 * Many periodic domains of different sizes, all with the same stencil,
 * storage and collision kind, advanced by one launch (the batched Taylor-
 * Green configuration; lettuce advances one Flow per Simulation and has no
 * counterpart). Domain b's populations are [Q][N_b] at element `offset` of
 * one pool; its relaxation times are per domain. */
typedef struct {
    int64_t offset;     /* element offset of the domain's [Q][rows * pitch] field in the pool */
    int32_t res[3];     /* lettuce resolution; unused trailing dims = 1 */
    int32_t pitch;      /* elements from one row (last lettuce dimension) to the next;
                           0 = the row length. With the 16-bit shifted formats every
                           row must be whole 32-bit words and the offset even: an odd
                           row length is stored with pitch = length + 1 (the pad
                           element is written and never read); other domains of these
                           formats are skipped with status bit 1. Population planes
                           are rows * pitch elements apart. */
    double tau;         /* BGK tau / TRT tau_plus */
    double tau_minus;   /* TRT */
} lgb_batch_domain;

typedef struct {
    int32_t domain;     /* index into the domain table */
    int32_t row_begin;  /* rows = cells along all but the last lettuce dimension */
    int32_t row_end;
    int32_t reserved;
} lgb_batch_tile;

typedef struct {
    int32_t abi_version;
    int32_t stencil;
    int32_t storage;
    int32_t collision;   /* LGB_NO_COLLISION, LGB_BGK or LGB_TRT */
    int32_t n_domains;
    int32_t n_tiles;
    int32_t threads;     /* threads per block (multiple of 32, <= 512) */
    int32_t blocks;      /* grid size: the blocks walk the tile table with a
                            grid stride (as many as the SMs hold, or one
                            block per tile) */
    const lgb_batch_domain *domains;  /* device copy of the domain table */
    const lgb_batch_tile *tiles;      /* device copy of the tile table */
    const void *f_in;    /* pool read this step */
    void *f_out;         /* pool written this step (pull pattern) */
    int64_t pool_elements;
    uint32_t *status;    /* optional; bit 0 non-finite density, bit 1 a tile
                            outside its domain or the pool, or a pitch the
                            domain's format does not accept (skipped) */
    const float *rates;  /* optional device table, 16-byte aligned, four floats
                            per domain: (float) (1 / tau), (float) (1 - 1 / tau),
                            (float) (1 / (2 tau)), (float) (1 / (2 tau_minus)),
                            each rounded once from the float64 value. With it the
                            float32 and 16-bit batches form no float64 quotient in
                            the kernel; NULL: formed per tile from tau (float64
                            batches always do). */
} lgb_batch_desc;

/* Host-only: cut every domain into tiles of whole rows holding about
 * `tile_cells` cells. With tiles == NULL only counts. Returns 0 and the
 * count in *n_tiles; fails if max_tiles is too small. */
int lgb_batch_plan(int32_t stencil, int32_t n_domains, const lgb_batch_domain *domains,
                   int32_t tile_cells, lgb_batch_tile *tiles, int32_t max_tiles,
                   int32_t *n_tiles);
/* One pull-pattern step (lettuce PRE_STREAMING) of every domain. */
int lgb_batched_step(const lgb_batch_desc *desc, void *stream);

/* Adjoint of one pull-pattern BGK step (lettuce PRE_STREAMING order):
 * lam = (d f_{n+1} / d f_n)^T lam_next, with f_n the state before the step.
 * float32 or float64 storage; lam must not alias f_n or lam_next. The
 * reverse pass of a differentiable rollout (torch autograd through
 * lettuce's step, lettuce/_simulation.py:241-305, computes the same
 * product); lettuce has no hand-written adjoint. */
int lgb_adjoint_step(int32_t stencil, int32_t storage, const int32_t *res, double tau,
                     const void *f_n, const void *lam_next, void *lam, void *stream);

/* Copy a population field between storage formats (for example float32
 * values into LGB_F16_SHIFTED storage and back). Replaces the dtype casts of
 * lettuce/_context.py:97-115 for the population field. */
int lgb_convert(int32_t stencil, int32_t src_storage, const void *src,
                int32_t dst_storage, void *dst, int64_t n_cells, void *stream);

/* The device address of page-locked, mapped host memory (memory from
 * cudaHostAlloc / cudaMallocHost, or registered with cudaHostRegister and
 * the mapped flag); fails for host memory the device cannot address (on a
 * host whose GPU reads pageable memory through the host page tables, such
 * as a Grace host, pageable memory is addressable too). With that address
 * lgb_convert moves a population field between host and device memory in
 * one kernel over the host link, converting the storage format on the way.
 * No lettuce counterpart: lettuce moves fields with torch copies
 * (lettuce/_flow.py:258-268, Context.convert_to_tensor). A kernel is used
 * because on a GB300 host the copy engines' first device-to-host transfer
 * after a period of GPU work runs at a tenth of the link rate, while kernel
 * stores to mapped host memory do not. */
int lgb_host_pointer(const void *host, void **device);

#ifdef __cplusplus
}
#endif
#endif
