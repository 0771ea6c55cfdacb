// Initial populations and the enstrophy observable on the device:
//
//   lgb_equilibrium  f = feq(rho, u) of broadcast density / velocity fields
//                    (lettuce/_flow.py:127-143 Flow.initialize with
//                    lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24),
//                    optionally the moments of that equilibrium only
//   lgb_init_fneq    f = feq(rho, u) - fneq(rho, u, grad u)
//                    (lettuce/_flow.py:341-367 initialize_f_neq, with the
//                    6th-order periodic differences of
//                    lettuce/util/utility.py:37-99)
//   lgb_enstrophy    sum over cells of |curl u|^2 from the same differences
//                    (lettuce/ext/_reporter/observable_reporter.py:45-67)
//
// This unit is compiled with -fmad=false: every product and sum below is
// rounded on its own, in the order lettuce's torch expressions evaluate
// them, so the float64 results stay within a few ulp of lettuce's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "lettuce_gb300.h"
#include "lgb_step.cuh"

namespace lgb {
int set_error(const char *msg);
}

namespace {

int init_fail(const char *fmt, const char *what, long long a = 0, long long b = 0) {
    char buf[512];
    snprintf(buf, sizeof(buf), fmt, what, a, b);
    return lgb::set_error(buf);
}

struct InitGrid {
    int d, q;
    uint32_t X, Y, Z, N;
    uint32_t ext[3];  // internal extents X, Y, Z
};

int init_grid(const char *what, int32_t stencil, const int32_t *res, InitGrid *g) {
    switch (stencil) {
    case LGB_D1Q3: g->d = 1; g->q = 3; break;
    case LGB_D2Q9: g->d = 2; g->q = 9; break;
    case LGB_D3Q15: g->d = 3; g->q = 15; break;
    case LGB_D3Q19: g->d = 3; g->q = 19; break;
    case LGB_D3Q27: g->d = 3; g->q = 27; break;
    default: return init_fail("%s: unknown stencil id %lld", what, stencil);
    }
    if (!res) return init_fail("%s: resolution pointer is NULL", what);
    uint64_t r[3] = {1, 1, 1};
    for (int i = 0; i < g->d; ++i) {
        if (res[i] <= 0) return init_fail("%s: resolution[%lld] = %lld must be positive", what, i, res[i]);
        r[3 - g->d + i] = (uint64_t)res[i];
    }
    const uint64_t n = r[0] * r[1] * r[2];
    if (n >= (1ull << 32))
        return init_fail("%s: grid of %lld cells exceeds the 2^32-1 cell limit", what, (long long)n);
    g->X = (uint32_t)r[0]; g->Y = (uint32_t)r[1]; g->Z = (uint32_t)r[2]; g->N = (uint32_t)n;
    g->ext[0] = g->X; g->ext[1] = g->Y; g->ext[2] = g->Z;
    return 0;
}

// cs^2 as lettuce's tables hold it: cs = 1 / sqrt(3) in float64, squared
inline double lettuce_cs2() {
    const double cs = 1.0 / std::sqrt(3.0);
    return cs * cs;
}

}  // namespace

namespace lgb {

// quadratic equilibrium of one population in lettuce's evaluation order:
// w * (rho * ((2 e.u - u.u) / (2 cs^2) + 0.5 (e.u / cs^2)^2 + 1))
template <class S, class R>
__device__ __forceinline__ R feq_lettuce_order(int q, R rho, const R (&u)[3], R uu, R two_cs2, R cs2) {
    R eu = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) eu = eu + R(S::e(q, d)) * u[d];
    const R a = eu / cs2;
    const R inner = rho * ((R(2) * eu - uu) / two_cs2 + R(0.5) * (a * a) + R(1));
    return R(S::w(q)) * inner;
}

template <class R>
__device__ __forceinline__ R dot3(const R (&u)[3], int D) {
    R uu = R(0);
    for (int d = 0; d < D; ++d) uu = uu + u[d] * u[d];
    return uu;
}

struct EqArgs {
    const void *rho;
    const void *u;
    int64_t rs[3];   // density strides, internal X, Y, Z
    int64_t us[4];   // velocity strides: component, internal X, Y, Z
    void *f;         // [Q][N] in the storage format, or NULL
    void *rho_out;   // [N] compute type, or NULL
    void *u_out;     // [D][N] compute type, or NULL
    uint32_t X, Y, Z, N;
    FastDiv divZ, divY;
    double cs2;
};

template <int SID, int ST>
__global__ void __launch_bounds__(256) equilibrium_kernel(EqArgs a) {
    using S = Stencil<SID>;
    using Sto = Storage<ST>;
    using R = typename Sto::R;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const uint32_t row = a.divZ.div(n), z = n - row * a.Z;
    const uint32_t x = a.divY.div(row), y = row - x * a.Y;
    const R *rho_p = static_cast<const R *>(a.rho);
    const R *u_p = static_cast<const R *>(a.u);
    const R rho = rho_p[x * a.rs[0] + y * a.rs[1] + z * a.rs[2]];
    R u[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int d = 0; d < S::D; ++d) u[d] = u_p[d * a.us[0] + x * a.us[1] + y * a.us[2] + z * a.us[3]];
    const R cs2 = R(a.cs2), two_cs2 = R(2.0 * a.cs2);
    const R uu = dot3(u, S::D);
    R f[S::Q];
#pragma unroll
    for (int q = 0; q < S::Q; ++q) f[q] = feq_lettuce_order<S>(q, rho, u, uu, two_cs2, cs2);
    if (a.f) {
        typename Sto::T *fo = static_cast<typename Sto::T *>(a.f);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) Sto::store(fo + (size_t)q * a.N + n, f[q], S::w(q));
    }
    if (a.rho_out) {
        // lettuce's Flow.rho / Flow.u of the field just set: sum over q,
        // then j / rho
        R r = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) r = r + f[q];
        static_cast<R *>(a.rho_out)[n] = r;
#pragma unroll
        for (int d = 0; d < S::D; ++d) {
            R j = R(0);
#pragma unroll
            for (int q = 0; q < S::Q; ++q) j = j + R(S::e(q, d)) * f[q];
            static_cast<R *>(a.u_out)[(size_t)d * a.N + n] = j / r;
        }
    }
}

// 6th-order central difference along internal axis `ax` of a periodic field
// v (lettuce/util/utility.py:37-99 with order 6 and dx = 1): the weights of
// the rolls by +3 ... -3 summed left to right
template <class R>
__device__ __forceinline__ R diff6(const R *v, const uint32_t (&c)[3], const uint32_t (&ext)[3],
                                   int ax) {
    const R wgt[6] = {R(-1.0 / 60.0), R(3.0 / 20.0), R(-3.0 / 4.0), R(3.0 / 4.0), R(-3.0 / 20.0),
                      R(1.0 / 60.0)};
    const int shift[6] = {3, 2, 1, -1, -2, -3};
    const uint32_t n_ax = ext[ax];
    R acc = R(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // roll by s reads the value at coordinate - s (periodic)
        uint32_t cc[3] = {c[0], c[1], c[2]};
        cc[ax] = (uint32_t)(((uint64_t)c[ax] + 3ull * n_ax - (uint64_t)(int64_t)shift[k]) % n_ax);
        const R term = wgt[k] * v[((size_t)cc[0] * ext[1] + cc[1]) * ext[2] + cc[2]];
        acc = k == 0 ? term : acc + term;
    }
    return acc;
}

struct FneqArgs {
    const void *rho;  // [N]
    const void *u;    // [D][N]
    void *f;          // [Q][N] storage format
    uint32_t ext[3];
    uint32_t N;
    FastDiv divZ, divY;
    double tau;
    double cs2;       // lettuce's cs^2 (float64)
    double cs2_f32;   // cs^2 rounded to float32 (the identity term of Q)
};

template <int SID, int ST>
__global__ void __launch_bounds__(256) init_fneq_kernel(FneqArgs a) {
    using S = Stencil<SID>;
    using Sto = Storage<ST>;
    using R = typename Sto::R;
    constexpr int D = S::D;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.N) return;
    const uint32_t row = a.divZ.div(n), cz = n - row * a.ext[2];
    const uint32_t cx = a.divY.div(row), cy = row - cx * a.ext[1];
    const uint32_t c[3] = {cx, cy, cz};
    const R *u_p = static_cast<const R *>(a.u);
    const R rho = static_cast<const R *>(a.rho)[n];
    R u[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int d = 0; d < D; ++d) u[d] = u_p[(size_t)d * a.N + n];
    // Pi_1[a][b] = tau rho (d_b u_a) / cs^2 (lettuce/_flow.py:355-356)
    const R t = R(a.tau) * rho;
    R pi[3][3];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
        for (int b = 0; b < D; ++b)
            pi[i][b] = (t * diff6(u_p + (size_t)i * a.N, c, a.ext, 3 - D + b)) / R(a.cs2);
    const R cs2 = R(a.cs2), two_cs2 = R(2.0 * a.cs2);
    const R iso = R(a.cs2_f32);
    const R uu = dot3(u, D);
    typename Sto::T *fo = static_cast<typename Sto::T *>(a.f);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        // Pi_1 : Q_q with Q_qab = e_qa e_qb - delta_ab cs^2 (:357-361)
        R pq = R(0);
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
            for (int b = 0; b < D; ++b) {
                const R qab = R(S::e(q, i) * S::e(q, b)) - (i == b ? iso : R(0));
                pq = (i == 0 && b == 0) ? pi[i][b] * qab : pq + pi[i][b] * qab;
            }
        const R fneq = R(S::w(q)) * pq;
        const R feq = feq_lettuce_order<S>(q, rho, u, uu, two_cs2, cs2);
        Sto::store(fo + (size_t)q * a.N + n, feq - fneq, S::w(q));
    }
}

constexpr int kEnsBlocks = 1216;
constexpr int kEnsThreads = 256;

__device__ __forceinline__ double block_sum(double v, double *smem) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? smem[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// squared vorticity of a velocity field [D][N] (D = 2 or 3), summed per
// block: 2-D (d_1 u_0 - d_0 u_1)^2; 3-D adds (d_1 u_2 - d_2 u_1)^2 and
// (d_2 u_0 - d_0 u_2)^2, d_b the difference along lettuce dimension b
template <class R>
__global__ void __launch_bounds__(kEnsThreads) enstrophy_partials_kernel(
    const R *u, int D, uint32_t X, uint32_t Y, uint32_t Z, uint32_t N, FastDiv divZ, FastDiv divY,
    double *partials) {
    __shared__ double smem[kEnsThreads / 32];
    const uint32_t ext[3] = {X, Y, Z};
    const int o = 3 - D;
    double acc = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t n = (uint32_t)i;
        const uint32_t row = divZ.div(n), cz = n - row * Z;
        const uint32_t cx = divY.div(row), cy = row - cx * Y;
        const uint32_t c[3] = {cx, cy, cz};
        const R *u0 = u, *u1 = u + N;
        const R w3 = diff6(u0, c, ext, o + 1) - diff6(u1, c, ext, o + 0);
        double s = (double)w3 * (double)w3;
        if (D == 3) {
            const R *u2 = u + 2 * (size_t)N;
            const R w1 = diff6(u2, c, ext, o + 1) - diff6(u1, c, ext, o + 2);
            const R w2 = diff6(u0, c, ext, o + 2) - diff6(u2, c, ext, o + 0);
            s += (double)w1 * (double)w1 + (double)w2 * (double)w2;
        }
        acc += s;
    }
    acc = block_sum(acc, smem);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kEnsThreads) sum_partials_kernel(const double *partials, int n,
                                                                   double *out) {
    __shared__ double smem[kEnsThreads / 32];
    double v = 0.0;
    for (int b = threadIdx.x; b < n; b += blockDim.x) v += partials[b];
    v = block_sum(v, smem);
    if (threadIdx.x == 0) out[0] = v;
}

}  // namespace lgb

namespace {

#define LGB_INIT_SWITCH(stencil, storage, CALL)                                      \
    switch (stencil) {                                                               \
    case LGB_D1Q3: switch (storage) { case 0: return CALL(LGB_D1Q3, 0); case 1: return CALL(LGB_D1Q3, 1); case 2: return CALL(LGB_D1Q3, 2); case 3: return CALL(LGB_D1Q3, 3); } break; \
    case LGB_D2Q9: switch (storage) { case 0: return CALL(LGB_D2Q9, 0); case 1: return CALL(LGB_D2Q9, 1); case 2: return CALL(LGB_D2Q9, 2); case 3: return CALL(LGB_D2Q9, 3); } break; \
    case LGB_D3Q15: switch (storage) { case 0: return CALL(LGB_D3Q15, 0); case 1: return CALL(LGB_D3Q15, 1); case 2: return CALL(LGB_D3Q15, 2); case 3: return CALL(LGB_D3Q15, 3); } break; \
    case LGB_D3Q19: switch (storage) { case 0: return CALL(LGB_D3Q19, 0); case 1: return CALL(LGB_D3Q19, 1); case 2: return CALL(LGB_D3Q19, 2); case 3: return CALL(LGB_D3Q19, 3); } break; \
    case LGB_D3Q27: switch (storage) { case 0: return CALL(LGB_D3Q27, 0); case 1: return CALL(LGB_D3Q27, 1); case 2: return CALL(LGB_D3Q27, 2); case 3: return CALL(LGB_D3Q27, 3); } break; \
    }

template <int SID, int ST>
cudaError_t launch_equilibrium(const lgb::EqArgs &a, cudaStream_t s) {
    lgb::equilibrium_kernel<SID, ST><<<(a.N + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

template <int SID, int ST>
cudaError_t launch_fneq(const lgb::FneqArgs &a, cudaStream_t s) {
    lgb::init_fneq_kernel<SID, ST><<<(a.N + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t equilibrium_dispatch(int stencil, int storage, const lgb::EqArgs &a, cudaStream_t s) {
#define CALL(SID, ST) launch_equilibrium<SID, ST>(a, s)
    LGB_INIT_SWITCH(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

cudaError_t fneq_dispatch(int stencil, int storage, const lgb::FneqArgs &a, cudaStream_t s) {
#define CALL(SID, ST) launch_fneq<SID, ST>(a, s)
    LGB_INIT_SWITCH(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

int cuda_error(const char *what, cudaError_t e) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return lgb::set_error(buf);
}

}  // namespace

extern "C" {

int lgb_equilibrium(int32_t stencil, int32_t storage, const int32_t *res, const void *rho,
                    const int64_t *rho_stride, const void *u, const int64_t *u_stride, void *f,
                    void *rho_out, void *u_out, void *stream) {
    const char *what = "lgb_equilibrium";
    InitGrid g;
    if (init_grid(what, stencil, res, &g)) return -1;
    if (storage < LGB_F64 || storage > LGB_BF16_SHIFTED)
        return init_fail("%s: unknown storage id %lld", what, storage);
    if (!rho || !u || !rho_stride || !u_stride) return init_fail("%s: NULL density or velocity", what);
    if (!f && !rho_out) return init_fail("%s: neither a field nor moments to write", what);
    if ((rho_out == nullptr) != (u_out == nullptr))
        return init_fail("%s: rho_out and u_out go together", what);
    lgb::EqArgs a;
    a.rho = rho; a.u = u; a.f = f; a.rho_out = rho_out; a.u_out = u_out;
    for (int i = 0; i < 3; ++i) a.rs[i] = 0;
    for (int i = 0; i < 4; ++i) a.us[i] = 0;
    const int off = 3 - g.d;
    for (int i = 0; i < g.d; ++i) {
        if (rho_stride[i] < 0 || u_stride[1 + i] < 0)
            return init_fail("%s: negative stride along dimension %lld", what, i);
        a.rs[off + i] = rho_stride[i];
        a.us[1 + off + i] = u_stride[1 + i];
    }
    if (u_stride[0] < 0) return init_fail("%s: negative component stride", what);
    a.us[0] = u_stride[0];
    a.X = g.X; a.Y = g.Y; a.Z = g.Z; a.N = g.N;
    a.divZ = lgb::FastDiv::make(g.Z);
    a.divY = lgb::FastDiv::make(g.Y);
    a.cs2 = lettuce_cs2();
    const cudaError_t e = equilibrium_dispatch(stencil, storage, a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error("lgb_equilibrium: launch failed", e);
    return 0;
}

int lgb_init_fneq(int32_t stencil, int32_t storage, const int32_t *res, const void *rho,
                  const void *u, double tau, void *f, void *stream) {
    const char *what = "lgb_init_fneq";
    InitGrid g;
    if (init_grid(what, stencil, res, &g)) return -1;
    if (storage < LGB_F64 || storage > LGB_BF16_SHIFTED)
        return init_fail("%s: unknown storage id %lld", what, storage);
    if (!rho || !u || !f) return init_fail("%s: NULL pointer", what);
    if (!(tau > 0.0) || !std::isfinite(tau)) return init_fail("%s: tau must be positive", what);
    if (g.d < 2) return init_fail("%s: the non-equilibrium initialisation is 2-D or 3-D", what);
    lgb::FneqArgs a;
    a.rho = rho; a.u = u; a.f = f;
    a.ext[0] = g.X; a.ext[1] = g.Y; a.ext[2] = g.Z;
    a.N = g.N;
    a.divZ = lgb::FastDiv::make(g.Z);
    a.divY = lgb::FastDiv::make(g.Y);
    a.tau = tau;
    a.cs2 = lettuce_cs2();
    a.cs2_f32 = (double)(float)a.cs2;
    const cudaError_t e = fneq_dispatch(stencil, storage, a, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error("lgb_init_fneq: launch failed", e);
    return 0;
}

int lgb_enstrophy(int32_t dims, int32_t precision, const int32_t *res, const void *u, double *out,
                  void *scratch, void *stream) {
    const char *what = "lgb_enstrophy";
    if (dims != 2 && dims != 3) return init_fail("%s: %lld dimensions (2 or 3)", what, dims);
    if (precision != LGB_F64 && precision != LGB_F32)
        return init_fail("%s: velocity precision %lld (LGB_F64 or LGB_F32)", what, precision);
    if (!u || !out || !scratch) return init_fail("%s: NULL pointer", what);
    InitGrid g;
    if (init_grid(what, dims == 2 ? LGB_D2Q9 : LGB_D3Q19, res, &g)) return -1;
    const lgb::FastDiv dz = lgb::FastDiv::make(g.Z), dy = lgb::FastDiv::make(g.Y);
    double *partials = static_cast<double *>(scratch);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (precision == LGB_F64)
        lgb::enstrophy_partials_kernel<double><<<lgb::kEnsBlocks, lgb::kEnsThreads, 0, s>>>(
            static_cast<const double *>(u), dims, g.X, g.Y, g.Z, g.N, dz, dy, partials);
    else
        lgb::enstrophy_partials_kernel<float><<<lgb::kEnsBlocks, lgb::kEnsThreads, 0, s>>>(
            static_cast<const float *>(u), dims, g.X, g.Y, g.Z, g.N, dz, dy, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error("lgb_enstrophy: launch failed", e);
    lgb::sum_partials_kernel<<<1, lgb::kEnsThreads, 0, s>>>(partials, lgb::kEnsBlocks, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error("lgb_enstrophy: launch failed", e);
    return 0;
}

}  // extern "C"
