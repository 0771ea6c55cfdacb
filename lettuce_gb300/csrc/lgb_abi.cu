// extern "C" entry points of liblettuce_gb300.so (declared in
// include/lettuce_gb300.h): argument validation, packing of the kernel
// parameter block, dispatch to the per-stencil instantiations, and the
// moment / reduction / conversion kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "lettuce_gb300.h"
#include "lgb_step.cuh"
#include "lgb_step_vec.cuh"

namespace {

thread_local std::string g_last_error;

int fail(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
int fail(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return -1;
}

}  // namespace

namespace lgb {
int set_error(const char *msg) {
    g_last_error = msg;
    return -1;
}
}  // namespace lgb

namespace {

int cuda_fail(cudaError_t e, const char *what) {
    return fail("%s: %s", what, cudaGetErrorString(e));
}

int stencil_dq(int s, int *d, int *q) {
    switch (s) {
    case LGB_D1Q3: *d = 1; *q = 3; return 0;
    case LGB_D2Q9: *d = 2; *q = 9; return 0;
    case LGB_D3Q15: *d = 3; *q = 15; return 0;
    case LGB_D3Q19: *d = 3; *q = 19; return 0;
    case LGB_D3Q27: *d = 3; *q = 27; return 0;
    }
    return -1;
}

struct Grid {
    int d, q;
    uint32_t X, Y, Z, N;
};

int make_grid(int stencil, const int32_t *res, Grid *g) {
    if (stencil_dq(stencil, &g->d, &g->q)) return fail("unknown stencil id %d", stencil);
    if (!res) return fail("resolution pointer is NULL");
    uint64_t r[3] = {1, 1, 1};
    for (int i = 0; i < g->d; ++i) {
        if (res[i] <= 0) return fail("resolution[%d] = %d must be positive", i, res[i]);
        r[3 - g->d + i] = (uint64_t)res[i];
    }
    const uint64_t n = r[0] * r[1] * r[2];
    if (n >= (1ull << 32)) return fail("grid of %llu cells exceeds the 2^32-1 cell limit",
                                       (unsigned long long)n);
    g->X = (uint32_t)r[0]; g->Y = (uint32_t)r[1]; g->Z = (uint32_t)r[2]; g->N = (uint32_t)n;
    return 0;
}

bool valid_storage(int s) { return s >= LGB_F64 && s <= LGB_BF16_SHIFTED; }

// per host thread and device: a second stream and the two events of a
// fork/join (per thread, so that concurrent callers do not reorder each
// other's events). Created on first use outside a stream capture.
struct AuxStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
thread_local AuxStream g_aux[64];

}  // namespace

namespace lgb {
cudaStream_t fork_aux(cudaStream_t s) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return nullptr;
    }
    AuxStream &a = g_aux[dev];
    if (!a.stream) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return nullptr;
        }
        cudaStream_t st = nullptr;
        cudaEvent_t ef = nullptr, ej = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ef, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ej, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (ef) cudaEventDestroy(ef);
            if (st) cudaStreamDestroy(st);
            return nullptr;
        }
        a.stream = st;
        a.fork = ef;
        a.join = ej;
    }
    if (cudaEventRecord(a.fork, s) != cudaSuccess ||
        cudaStreamWaitEvent(a.stream, a.fork, 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.stream;
}

cudaError_t join_aux(cudaStream_t s, cudaStream_t aux) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    AuxStream &a = g_aux[dev];
    if (aux != a.stream) return cudaErrorInvalidValue;
    e = cudaEventRecord(a.join, aux);
    if (e != cudaSuccess) return e;
    return cudaStreamWaitEvent(s, a.join, 0);
}
}  // namespace lgb

namespace {

cudaError_t dispatch_step(int stencil, int storage, int coll, int pat, bool masked,
                          const lgb::StepParams &p, cudaStream_t s) {
#define LGB_PART_CALL(name, st)                                                             \
    (!masked ? lgb::name##_plain_##st(coll, pat, p, s)                                      \
             : lgb::pulling_pattern(pat) ? lgb::name##_masked_pull_##st(coll, pat, p, s)   \
                                         : lgb::name##_masked_rest_##st(coll, pat, p, s))
#define LGB_STORAGE_SWITCH(name)                                                            \
    switch (storage) {                                                                      \
    case 0: return LGB_PART_CALL(name, s0);                                                 \
    case 1: return LGB_PART_CALL(name, s1);                                                 \
    case 2: return LGB_PART_CALL(name, s2);                                                 \
    case 3: return LGB_PART_CALL(name, s3);                                                 \
    }                                                                                       \
    return cudaErrorInvalidValue;
    const bool ext = coll == lgb::LGB_BGK_FORCED || coll == LGB_REGULARIZED ||
                     coll == LGB_SMAGORINSKY || coll == LGB_MRT;
    if (ext) {
        switch (stencil) {
        case LGB_D1Q3: LGB_STORAGE_SWITCH(stepx_d1q3)
        case LGB_D2Q9: LGB_STORAGE_SWITCH(stepx_d2q9)
        case LGB_D3Q15: LGB_STORAGE_SWITCH(stepx_d3q15)
        case LGB_D3Q19: LGB_STORAGE_SWITCH(stepx_d3q19)
        case LGB_D3Q27: LGB_STORAGE_SWITCH(stepx_d3q27)
        }
        return cudaErrorInvalidValue;
    }
    switch (stencil) {
    case LGB_D1Q3: LGB_STORAGE_SWITCH(step_d1q3)
    case LGB_D2Q9: LGB_STORAGE_SWITCH(step_d2q9)
    case LGB_D3Q15: LGB_STORAGE_SWITCH(step_d3q15)
    case LGB_D3Q19: LGB_STORAGE_SWITCH(step_d3q19)
    case LGB_D3Q27: LGB_STORAGE_SWITCH(step_d3q27)
    }
#undef LGB_STORAGE_SWITCH
#undef LGB_PART_CALL
    return cudaErrorInvalidValue;
}

// the two-cell kernel of the 16-bit storages: no boundaries, BGK / TRT /
// no collision, an even row length and one of its five patterns
bool use_vec2(int storage, int coll, int pat, bool masked, uint32_t Z) {
    return (storage == LGB_F16_SHIFTED || storage == LGB_BF16_SHIFTED) && !masked &&
           (coll == LGB_NO_COLLISION || coll == LGB_BGK || coll == LGB_TRT) && Z % 2 == 0 &&
           (pat == LGB_PULL || pat == LGB_PUSH || pat == LGB_LOCAL || pat == LGB_AA_EVEN ||
            pat == LGB_AA_ODD);
}

cudaError_t dispatch_step_vec2(int stencil, int storage, int coll, int pat,
                               const lgb::StepParams &p, cudaStream_t s) {
#define LGB_VEC_SWITCH(name)                                                \
    return storage == LGB_F16_SHIFTED ? lgb::name##_s2(coll, pat, p, s)     \
                                      : lgb::name##_s3(coll, pat, p, s);
    switch (stencil) {
    case LGB_D1Q3: LGB_VEC_SWITCH(step_vec2_d1q3)
    case LGB_D2Q9: LGB_VEC_SWITCH(step_vec2_d2q9)
    case LGB_D3Q15: LGB_VEC_SWITCH(step_vec2_d3q15)
    case LGB_D3Q19: LGB_VEC_SWITCH(step_vec2_d3q19)
    case LGB_D3Q27: LGB_VEC_SWITCH(step_vec2_d3q27)
    }
#undef LGB_VEC_SWITCH
    return cudaErrorInvalidValue;
}

// ----------------------------------------------------------------------------
// moments

template <int SID, int ST, bool AA>
__global__ void __launch_bounds__(256) moments_kernel(const void *fv, uint32_t X, uint32_t Y,
                                                      uint32_t Z, uint32_t N, lgb::FastDiv divZ,
                                                      lgb::FastDiv divY, void *rho_v, void *u_v) {
    using S = lgb::Stencil<SID>;
    using Sto = lgb::Storage<ST>;
    using R = typename Sto::R;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    lgb::StepParams p;
    p.X = X; p.Y = Y; p.Z = Z; p.N = N;
    const uint32_t row = divZ.div(n), z = n - row * Z;
    const uint32_t x = divY.div(row), y = row - x * Y;
    lgb::Nbr c;
    c.set(x, y, z, p);
    R f[S::Q];
    lgb::load_cell<S, Sto, AA ? lgb::LOAD_AA_ODD : lgb::LOAD_OWN, false>(
        p, static_cast<const typename Sto::T *>(fv), c, n, 0u, f);
    R rho, u[3];
    lgb::cell_moments<S>(f, rho, u);
    static_cast<R *>(rho_v)[n] = rho;
#pragma unroll
    for (int d = 0; d < S::D; ++d) static_cast<R *>(u_v)[(size_t)d * N + n] = u[d];
}

template <int SID, int ST>
cudaError_t launch_moments(const Grid &g, const void *f, int aa, void *rho, void *u, cudaStream_t s) {
    const unsigned blocks = (g.N + 255) / 256;
    const lgb::FastDiv dz = lgb::FastDiv::make(g.Z), dy = lgb::FastDiv::make(g.Y);
    if (aa)
        moments_kernel<SID, ST, true><<<blocks, 256, 0, s>>>(f, g.X, g.Y, g.Z, g.N, dz, dy, rho, u);
    else
        moments_kernel<SID, ST, false><<<blocks, 256, 0, s>>>(f, g.X, g.Y, g.Z, g.N, dz, dy, rho, u);
    return cudaGetLastError();
}

// ----------------------------------------------------------------------------
// float64 reductions: grid-stride partials per block into scratch, then a
// single block folds the partials in a fixed order (deterministic result)

constexpr int kReduceBlocks = 1216;  // 152 SMs x 8
constexpr int kReduceThreads = 256;

struct ReduceBox {
    uint32_t lo[3], hi[3];  // internal X, Y, Z
};

__device__ __forceinline__ void block_fold(double (&v)[LGB_REDUCE_FIELDS], double *smem) {
    // warp shuffles, then one value per warp through shared memory
#pragma unroll
    for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_down_sync(0xffffffffu, v[i], o);
            v[i] = (i == 2) ? fmax(v[i], w) : v[i] + w;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) smem[warp * LGB_REDUCE_FIELDS + i] = v[i];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) v[i] = lane < nw ? smem[lane * LGB_REDUCE_FIELDS + i] : (i == 2 ? 0.0 : 0.0);
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double w = __shfl_down_sync(0xffffffffu, v[i], o);
                v[i] = (i == 2) ? fmax(v[i], w) : v[i] + w;
            }
        }
    }
}

template <int SID, int ST, bool AA>
__global__ void __launch_bounds__(kReduceThreads) reduce_partials_kernel(
    const void *fv, uint32_t X, uint32_t Y, uint32_t Z, uint32_t N, lgb::FastDiv divZ,
    lgb::FastDiv divY, ReduceBox box, const uint8_t *mask, double *partials) {
    using S = lgb::Stencil<SID>;
    using Sto = lgb::Storage<ST>;
    using R = typename Sto::R;
    __shared__ double smem[(kReduceThreads / 32) * LGB_REDUCE_FIELDS];
    lgb::StepParams p;
    p.X = X; p.Y = Y; p.Z = Z; p.N = N;
    double v[LGB_REDUCE_FIELDS] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t n = (uint32_t)i;
        const uint32_t row = divZ.div(n), z = n - row * Z;
        const uint32_t x = divY.div(row), y = row - x * Y;
        if (x < box.lo[0] || x >= box.hi[0] || y < box.lo[1] || y >= box.hi[1] || z < box.lo[2] ||
            z >= box.hi[2])
            continue;
        lgb::Nbr c;
        c.set(x, y, z, p);
        R f[S::Q];
        lgb::load_cell<S, Sto, AA ? lgb::LOAD_AA_ODD : lgb::LOAD_OWN, false>(
            p, static_cast<const typename Sto::T *>(fv), c, n, 0u, f);
        double rho = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int q = 0; q < S::Q; ++q) {
            const double fq = (double)f[q];
            rho += fq;
#pragma unroll
            for (int d = 0; d < S::D; ++d) j[d] += (double)S::e(q, d) * fq;
        }
        if (!isfinite(rho)) {
            v[3] += 1.0;
            continue;
        }
        double uu = 0.0;
#pragma unroll
        for (int d = 0; d < S::D; ++d) uu += (j[d] / rho) * (j[d] / rho);
        v[0] += rho;
        v[1] += 0.5 * uu;
        v[2] = fmax(v[2], uu);
        if (mask && mask[n]) v[4] += rho;
    }
    block_fold(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) partials[blockIdx.x * LGB_REDUCE_FIELDS + i] = v[i];
    }
}

__global__ void __launch_bounds__(kReduceThreads) reduce_final_kernel(const double *partials, int nblocks,
                                                                      double *out) {
    __shared__ double smem[(kReduceThreads / 32) * LGB_REDUCE_FIELDS];
    double v[LGB_REDUCE_FIELDS] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) {
            const double w = partials[b * LGB_REDUCE_FIELDS + i];
            v[i] = (i == 2) ? fmax(v[i], w) : v[i] + w;
        }
    }
    block_fold(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < LGB_REDUCE_FIELDS; ++i) out[i] = v[i];
    }
}

template <int SID, int ST>
cudaError_t launch_reduce(const Grid &g, const void *f, int aa, const ReduceBox &box,
                          const uint8_t *mask, double *out, double *partials, cudaStream_t s) {
    const lgb::FastDiv dz = lgb::FastDiv::make(g.Z), dy = lgb::FastDiv::make(g.Y);
    if (aa)
        reduce_partials_kernel<SID, ST, true><<<kReduceBlocks, kReduceThreads, 0, s>>>(
            f, g.X, g.Y, g.Z, g.N, dz, dy, box, mask, partials);
    else
        reduce_partials_kernel<SID, ST, false><<<kReduceBlocks, kReduceThreads, 0, s>>>(
            f, g.X, g.Y, g.Z, g.N, dz, dy, box, mask, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_final_kernel<<<1, kReduceThreads, 0, s>>>(partials, kReduceBlocks, out);
    return cudaGetLastError();
}

// ----------------------------------------------------------------------------
// storage conversion

template <int SID, int SRC, int DST>
__global__ void __launch_bounds__(256) convert_kernel(const void *src, void *dst, uint64_t n_cells) {
    using S = lgb::Stencil<SID>;
    const uint64_t total = n_cells * (uint64_t)S::Q;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i / n_cells);
        double w = 0.0;
#pragma unroll
        for (int k = 0; k < S::Q; ++k)
            if (k == q) w = S::w(k);
        const auto v = lgb::Storage<SRC>::load_plain(static_cast<const typename lgb::Storage<SRC>::T *>(src) + i, w);
        lgb::Storage<DST>::store(static_cast<typename lgb::Storage<DST>::T *>(dst) + i,
                                 (typename lgb::Storage<DST>::R)v, w);
    }
}

template <int SID, int SRC>
cudaError_t launch_convert_dst(int dst_st, const void *src, void *dst, uint64_t n, cudaStream_t s) {
    const unsigned blocks = 152 * 16;
    switch (dst_st) {
    case LGB_F64: convert_kernel<SID, SRC, LGB_F64><<<blocks, 256, 0, s>>>(src, dst, n); break;
    case LGB_F32: convert_kernel<SID, SRC, LGB_F32><<<blocks, 256, 0, s>>>(src, dst, n); break;
    case LGB_F16_SHIFTED: convert_kernel<SID, SRC, LGB_F16_SHIFTED><<<blocks, 256, 0, s>>>(src, dst, n); break;
    case LGB_BF16_SHIFTED: convert_kernel<SID, SRC, LGB_BF16_SHIFTED><<<blocks, 256, 0, s>>>(src, dst, n); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int SID>
cudaError_t launch_convert(int src_st, const void *src, int dst_st, void *dst, uint64_t n, cudaStream_t s) {
    switch (src_st) {
    case LGB_F64: return launch_convert_dst<SID, LGB_F64>(dst_st, src, dst, n, s);
    case LGB_F32: return launch_convert_dst<SID, LGB_F32>(dst_st, src, dst, n, s);
    case LGB_F16_SHIFTED: return launch_convert_dst<SID, LGB_F16_SHIFTED>(dst_st, src, dst, n, s);
    case LGB_BF16_SHIFTED: return launch_convert_dst<SID, LGB_BF16_SHIFTED>(dst_st, src, dst, n, s);
    }
    return cudaErrorInvalidValue;
}

// Momentum exchange of bounce-back links (halfway_bounce_back_boundary.py:
// 211-218, linear_interpolated_bounce_back_boundary.py:104-126):
// F = sum_k (g_k + b_k) e_{q_k}, g_k = f*_{q_k}(n_k) from the post-collision
// field, b_k the bounced value (link_val[j_k], or g_k for a halfway link),
// over the (q_k, n_k, j_k) triplets; a full-way link (bit 31 of j_k) counts
// 2 b_k e_{q_k}, b_k its streamed value (fullway_bounce_back_boundary.py:
// 163-178). Block b reduces links
// [b * 256, b * 256 + 256) into partial[3 b .. 3 b + 2] by a fixed tree;
// link_force_total adds the partial sums in a fixed order, so the result
// does not depend on scheduling. Entries outside the field or the value
// table count zero.
template <int SID, int ST>
__global__ void __launch_bounds__(LGB_LINK_FORCE_BLOCK)
link_force_partial(const void *f, uint64_t n_cells, const uint32_t *links, int64_t n_links,
                   const void *vals, int64_t n_vals, double *partial) {
    using S = lgb::Stencil<SID>;
    using Sto = lgb::Storage<ST>;
    __shared__ double part[3][LGB_LINK_FORCE_BLOCK];
    double F[3] = {0.0, 0.0, 0.0};
    const int64_t k = blockIdx.x * (int64_t)LGB_LINK_FORCE_BLOCK + threadIdx.x;
    if (k < n_links) {
        const uint32_t q = links[3 * k], n = links[3 * k + 1], jj = links[3 * k + 2];
        // jj: 0xffffffff = halfway; bit 31 set = full-way (2 b e_q, b the
        // streamed value in entry jj & 0x7fffffff); else interpolated
        const bool halfway = jj == 0xffffffffu;
        const bool fullway = !halfway && (jj & 0x80000000u);
        const uint32_t j = jj & 0x7fffffffu;
        bool ok = q < (uint32_t)S::Q && (uint64_t)n < n_cells;
        if (!halfway && (!vals || (int64_t)j >= n_vals)) ok = false;
        if (ok) {
            double w = 0.0;
            int e[3] = {0, 0, 0};
#pragma unroll
            for (int i = 0; i < S::Q; ++i) {
                if ((uint32_t)i == q) {
                    w = S::w(i);
#pragma unroll
                    for (int d = 0; d < S::D; ++d) e[d] = S::e(i, d);
                }
            }
            const double v = (double)Sto::load_plain(
                static_cast<const typename Sto::T *>(f) + (uint64_t)q * n_cells + n, w);
            const double b = halfway ? v
                                     : (double)Sto::load_plain(
                                           static_cast<const typename Sto::T *>(vals) + j, w);
            const double m = fullway ? 2.0 * b : v + b;
#pragma unroll
            for (int d = 0; d < 3; ++d) F[d] = m * (double)e[d];
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) part[d][threadIdx.x] = F[d];
    __syncthreads();
    for (int h = LGB_LINK_FORCE_BLOCK / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
#pragma unroll
            for (int d = 0; d < 3; ++d) part[d][threadIdx.x] += part[d][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x < 3) partial[3 * blockIdx.x + threadIdx.x] = part[threadIdx.x][0];
}

__global__ void __launch_bounds__(LGB_LINK_FORCE_BLOCK)
link_force_total(const double *partial, int64_t n_blocks, double *out) {
    __shared__ double part[3][LGB_LINK_FORCE_BLOCK];
    double F[3] = {0.0, 0.0, 0.0};
    for (int64_t b = threadIdx.x; b < n_blocks; b += LGB_LINK_FORCE_BLOCK) {
#pragma unroll
        for (int d = 0; d < 3; ++d) F[d] += partial[3 * b + d];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) part[d][threadIdx.x] = F[d];
    __syncthreads();
    for (int h = LGB_LINK_FORCE_BLOCK / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
#pragma unroll
            for (int d = 0; d < 3; ++d) part[d][threadIdx.x] += part[d][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x < 3) out[threadIdx.x] = part[threadIdx.x][0];
}

template <int SID, int ST>
cudaError_t launch_link_force_ss(const void *f, uint64_t n_cells, const uint32_t *links,
                                 int64_t n_links, const void *vals, int64_t n_vals, double *out,
                                 double *scratch, cudaStream_t s) {
    const int64_t blocks = (n_links + LGB_LINK_FORCE_BLOCK - 1) / LGB_LINK_FORCE_BLOCK;
    if (blocks > 0) {
        link_force_partial<SID, ST><<<(unsigned)blocks, LGB_LINK_FORCE_BLOCK, 0, s>>>(
            f, n_cells, links, n_links, vals, n_vals, scratch);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    link_force_total<<<1, LGB_LINK_FORCE_BLOCK, 0, s>>>(scratch, blocks, out);
    return cudaGetLastError();
}

// The interpolated bounce-back values of one step
// (linear_interpolated_bounce_back_boundary.py:55-96, in the EbbSimulation
// order: the links read the post-collision field f* and, for d < 1/2, the
// streamed value f_q(n) = f*_q(n - e_q)); one thread per link, computed in
// the step's arithmetic type and stored in the field's storage format (the
// table holds one storage element per link). Links outside the field are
// skipped.
template <int SID, int ST>
__global__ void __launch_bounds__(256) link_value_kernel(const void *f, uint32_t X, uint32_t Y,
                                                         uint32_t Z, const uint32_t *pairs,
                                                         const double *dist, int64_t n_links,
                                                         void *vals) {
    using S = lgb::Stencil<SID>;
    using Sto = lgb::Storage<ST>;
    using R = typename Sto::R;
    const uint64_t N = (uint64_t)X * Y * Z;
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n_links) return;
    const uint32_t q = pairs[2 * k], n = pairs[2 * k + 1];
    if (q >= (uint32_t)S::Q || (uint64_t)n >= N) return;
    double w = 0.0;
    int qo = 0, ex = 0, ey = 0, ez = 0;
#pragma unroll
    for (int i = 0; i < S::Q; ++i) {
        if ((uint32_t)i == q) {
            w = S::w(i);
            qo = S::opp(i);
            ex = lgb::ix<S>(i);
            ey = lgb::iy<S>(i);
            ez = lgb::iz<S>(i);
        }
    }
    const typename Sto::T *fp = static_cast<const typename Sto::T *>(f);
    const R g = Sto::load_plain(fp + (uint64_t)q * N + n, w);
    const R d = (R)dist[k];
    R v;
    if (d < R(0)) {
        v = g;
    } else if (d < R(0.5)) {
        const uint32_t z = n % Z, row = n / Z, y = row % Y, x = row / Y;
        const uint32_t xs = (x + X - (uint32_t)(ex + 1) + 1) % X;
        const uint32_t ys = (y + Y - (uint32_t)(ey + 1) + 1) % Y;
        const uint32_t zs = (z + Z - (uint32_t)(ez + 1) + 1) % Z;
        const R streamed = Sto::load_plain(fp + (uint64_t)q * N + ((uint64_t)xs * Y + ys) * Z + zs, w);
        v = R(2) * d * g + (R(1) - R(2) * d) * streamed;
    } else {
        const R go = Sto::load_plain(fp + (uint64_t)qo * N + n, w);
        v = (R(1) / (R(2) * d)) * g + (R(1) - R(1) / (R(2) * d)) * go;
    }
    Sto::store(static_cast<typename Sto::T *>(vals) + k, v, w);
}

template <int SID, int ST>
cudaError_t launch_link_values_ss(const void *f, const Grid &g, const uint32_t *pairs,
                                  const double *dist, int64_t n_links, void *vals,
                                  cudaStream_t s) {
    const unsigned blocks = (unsigned)((n_links + 255) / 256);
    link_value_kernel<SID, ST><<<blocks, 256, 0, s>>>(f, g.X, g.Y, g.Z, pairs, dist, n_links,
                                                      vals);
    return cudaGetLastError();
}

// stencil x storage switch for the templated helpers above
#define LGB_SWITCH_SS(stencil, storage, CALL)                                        \
    switch (stencil) {                                                               \
    case LGB_D1Q3: switch (storage) { case 0: return CALL(LGB_D1Q3, 0); case 1: return CALL(LGB_D1Q3, 1); case 2: return CALL(LGB_D1Q3, 2); case 3: return CALL(LGB_D1Q3, 3); } break; \
    case LGB_D2Q9: switch (storage) { case 0: return CALL(LGB_D2Q9, 0); case 1: return CALL(LGB_D2Q9, 1); case 2: return CALL(LGB_D2Q9, 2); case 3: return CALL(LGB_D2Q9, 3); } break; \
    case LGB_D3Q15: switch (storage) { case 0: return CALL(LGB_D3Q15, 0); case 1: return CALL(LGB_D3Q15, 1); case 2: return CALL(LGB_D3Q15, 2); case 3: return CALL(LGB_D3Q15, 3); } break; \
    case LGB_D3Q19: switch (storage) { case 0: return CALL(LGB_D3Q19, 0); case 1: return CALL(LGB_D3Q19, 1); case 2: return CALL(LGB_D3Q19, 2); case 3: return CALL(LGB_D3Q19, 3); } break; \
    case LGB_D3Q27: switch (storage) { case 0: return CALL(LGB_D3Q27, 0); case 1: return CALL(LGB_D3Q27, 1); case 2: return CALL(LGB_D3Q27, 2); case 3: return CALL(LGB_D3Q27, 3); } break; \
    }

cudaError_t launch_link_force(int stencil, int storage, const void *f, uint64_t n_cells,
                              const uint32_t *links, int64_t n_links, const void *vals,
                              int64_t n_vals, double *out, double *scratch, cudaStream_t s) {
#define CALL(SID, ST) \
    launch_link_force_ss<SID, ST>(f, n_cells, links, n_links, vals, n_vals, out, scratch, s)
    LGB_SWITCH_SS(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

cudaError_t launch_link_values(int stencil, int storage, const void *f, const Grid &g,
                               const uint32_t *pairs, const double *dist, int64_t n_links,
                               void *vals, cudaStream_t s) {
#define CALL(SID, ST) launch_link_values_ss<SID, ST>(f, g, pairs, dist, n_links, vals, s)
    LGB_SWITCH_SS(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

cudaError_t moments_dispatch(int stencil, int storage, const Grid &g, const void *f, int aa,
                             void *rho, void *u, cudaStream_t s) {
#define CALL(SID, ST) launch_moments<SID, ST>(g, f, aa, rho, u, s)
    LGB_SWITCH_SS(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

cudaError_t reduce_dispatch(int stencil, int storage, const Grid &g, const void *f, int aa,
                            const ReduceBox &box, const uint8_t *mask, double *out,
                            double *partials, cudaStream_t s) {
#define CALL(SID, ST) launch_reduce<SID, ST>(g, f, aa, box, mask, out, partials, s)
    LGB_SWITCH_SS(stencil, storage, CALL)
#undef CALL
    return cudaErrorInvalidValue;
}

cudaError_t convert_dispatch(int stencil, int src_st, const void *src, int dst_st, void *dst,
                             uint64_t n, cudaStream_t s) {
    switch (stencil) {
    case LGB_D1Q3: return launch_convert<LGB_D1Q3>(src_st, src, dst_st, dst, n, s);
    case LGB_D2Q9: return launch_convert<LGB_D2Q9>(src_st, src, dst_st, dst, n, s);
    case LGB_D3Q15: return launch_convert<LGB_D3Q15>(src_st, src, dst_st, dst, n, s);
    case LGB_D3Q19: return launch_convert<LGB_D3Q19>(src_st, src, dst_st, dst, n, s);
    case LGB_D3Q27: return launch_convert<LGB_D3Q27>(src_st, src, dst_st, dst, n, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

extern "C" {

int lgb_abi_version(void) { return LGB_ABI_VERSION; }

const char *lgb_last_error(void) { return g_last_error.c_str(); }

int lgb_step(const lgb_step_desc *d, void *stream) {
    if (!d) return fail("lgb_step: descriptor is NULL");
    if (d->abi_version != LGB_ABI_VERSION)
        return fail("lgb_step: descriptor ABI version %d, library %d", d->abi_version, LGB_ABI_VERSION);
    if (d->options & ~(LGB_OPT_ONE_CELL | LGB_OPT_PUSH_GUARD))
        return fail("lgb_step: unknown option bits 0x%x", (unsigned)d->options);
    Grid g;
    if (make_grid(d->stencil, d->res, &g)) return -1;
    if (!valid_storage(d->storage)) return fail("lgb_step: unknown storage id %d", d->storage);
    if (d->collision < LGB_NO_COLLISION || d->collision > LGB_MRT)
        return fail("lgb_step: unknown collision id %d", d->collision);
    if (d->collision == LGB_MRT) {
        if (!d->mrt_tables) return fail("lgb_step: the MRT collision needs its tables");
        if (d->mrt_equilibrium < LGB_MRT_EQ_GENERIC || d->mrt_equilibrium > LGB_MRT_EQ_HERMITE)
            return fail("lgb_step: unknown MRT equilibrium %d", d->mrt_equilibrium);
        if ((d->mrt_equilibrium == LGB_MRT_EQ_DELLAR || d->mrt_equilibrium == LGB_MRT_EQ_LALLEMAND) &&
            d->stencil != LGB_D2Q9)
            return fail("lgb_step: the Dellar and Lallemand moment bases are D2Q9 bases");
        if (d->mrt_equilibrium == LGB_MRT_EQ_HERMITE && d->stencil != LGB_D3Q27)
            return fail("lgb_step: the Hermite moment basis is a D3Q27 basis");
        const int Q = g.q;
        for (int i = 0; i < Q; ++i) {
            const double s = d->mrt_tables[2 * Q * Q + i];
            if (!(s != 0.0) || !std::isfinite(s))
                return fail("lgb_step: MRT relaxation time %d is %g", i, s);
        }
    }
    if (d->force < LGB_FORCE_NONE || d->force > LGB_FORCE_SHAN_CHEN)
        return fail("lgb_step: unknown force id %d", d->force);
    if (d->force != LGB_FORCE_NONE && d->collision != LGB_BGK && d->collision != LGB_SMAGORINSKY)
        return fail("lgb_step: a body force needs the BGK or Smagorinsky collision");
    if (d->force != LGB_FORCE_NONE && !(d->force_tau > 0.0))
        return fail("lgb_step: the force's tau must be positive (got %g)", d->force_tau);
    if (d->collision == LGB_KBC && !(d->stencil == LGB_D2Q9 || d->stencil == LGB_D3Q27))
        return fail("lgb_step: KBC collision is only defined for D2Q9 and D3Q27");
    if (d->pattern < LGB_PULL || d->pattern > LGB_AA_UNPACK)
        return fail("lgb_step: unknown access pattern %d", d->pattern);
    if (!d->f_in || !d->f_out) return fail("lgb_step: population pointer is NULL");
    const bool in_place_ok = d->pattern == LGB_LOCAL || d->pattern == LGB_AA_EVEN || d->pattern == LGB_AA_ODD;
    if (!in_place_ok && d->f_in == d->f_out)
        return fail("lgb_step: pattern %d needs distinct input and output fields", d->pattern);
    if (d->collision != LGB_NO_COLLISION && d->collision != LGB_MRT && !(d->tau > 0.0))
        return fail("lgb_step: relaxation time must be positive (got %g)", d->tau);
    if (d->collision == LGB_TRT && !(d->tau_minus > 0.0))
        return fail("lgb_step: TRT tau_minus must be positive (got %g)", d->tau_minus);

    lgb::StepParams p;
    std::memset(&p, 0, sizeof(p));
    p.f_in = d->f_in;
    p.f_out = d->f_out;
    p.X = g.X; p.Y = g.Y; p.Z = g.Z; p.N = g.N;
    p.divZ = lgb::FastDiv::make(g.Z);
    p.divY = lgb::FastDiv::make(g.Y);
    p.cp.omega = 1.0 / d->tau;
    p.cp.inv_2tp = 1.0 / (2.0 * d->tau);
    p.cp.inv_2tm = d->collision == LGB_TRT ? 1.0 / (2.0 * d->tau_minus) : 0.0;
    p.cp.beta = 1.0 / (2.0 * d->tau);
    lgb::set_float_rates(p.cp);
    p.cp.tau = d->tau;
    p.cp.smag_c2 = d->smagorinsky_constant * d->smagorinsky_constant;
    p.mrt_host = d->mrt_tables;
    p.mrt_eq = d->mrt_equilibrium;
    if (d->force != LGB_FORCE_NONE) {
        for (int i = 0; i < 3; ++i) p.cp.accel[i] = i < g.d ? d->accel[i] : 0.0;
        p.cp.ueq_scale = d->force == LGB_FORCE_GUO ? 0.5 : d->force_tau;
        p.cp.src_scale = d->force == LGB_FORCE_GUO ? 1.0 - 1.0 / (2.0 * d->force_tau) : 0.0;
    }
    p.status = d->status;
    p.abb_k = -1;
    const bool masked = d->flags != nullptr;
    if (masked && d->pattern == LGB_AA_UNPACK)
        return fail("lgb_step: AA_UNPACK takes no boundary flags");
    if (masked) {
        if (d->n_sub < 1 || d->n_sub > LGB_MAX_SUBSTEPS)
            return fail("lgb_step: %d substeps (1..%d supported)", d->n_sub, LGB_MAX_SUBSTEPS);
        if (d->collision_index < 0 || d->collision_index >= d->n_sub ||
            d->sub[d->collision_index].kind != LGB_SUB_COLLISION)
            return fail("lgb_step: collision_index %d does not name the collision substep",
                        d->collision_index);
        p.flags = d->flags;
        p.nsb = d->no_stream_bits;
        p.has_nsm = d->no_stream_bits != nullptr;
        p.push_guard = (d->options & LGB_OPT_PUSH_GUARD) != 0;
        if (p.has_nsm && (d->pattern == LGB_AA_EVEN || d->pattern == LGB_AA_ODD))
            return fail("lgb_step: no-streaming masks are not supported by the AA pattern");
        p.n_sub = d->n_sub;
        p.coll_idx = d->collision_index;
        const int off = 3 - g.d;
        for (int k = 0; k < d->n_sub; ++k) {
            const lgb_substep &s = d->sub[k];
            lgb::SubParams &t = p.sub[k];
            if (s.kind < LGB_SUB_COLLISION || s.kind > LGB_SUB_PARTIALLY_SATURATED)
                return fail("lgb_step: substep %d has unknown kind %d", k, s.kind);
            if (s.kind == LGB_SUB_COLLISION && k != d->collision_index)
                return fail("lgb_step: substep %d is a second collision", k);
            t.kind = s.kind;
            if (s.kind == LGB_SUB_EQUILIBRIUM_PU) {
                if (!s.rho || !s.u) return fail("lgb_step: equilibrium substep %d lacks rho/u", k);
                t.rho = s.rho;
                t.u = s.u;
                t.us[0] = s.u_stride[0];
                for (int i = 0; i < g.d; ++i) {
                    t.rs[off + i] = s.rho_stride[i];
                    t.us[1 + off + i] = s.u_stride[1 + i];
                }
            }
            if (s.kind == LGB_SUB_PARTIALLY_SATURATED) {
                if (!(s.param[0] > 0.0))
                    return fail("lgb_step: partially saturated substep %d needs tau > 0", k);
                t.param[0] = s.param[0];
                t.param[1] = s.param[1];
            }
            if (s.kind == LGB_SUB_ANTI_BOUNCE_BACK || s.kind == LGB_SUB_EQUILIBRIUM_OUTLET_P) {
                if (p.abb_k >= 0) return fail("lgb_step: more than one outlet-plane substep");
                p.abb_kind = s.kind;
                p.abb_rho = s.param[0];
                if (s.axis < 0 || s.axis >= g.d || (s.sign != 1 && s.sign != -1))
                    return fail("lgb_step: outlet direction (axis %d, sign %d) invalid", s.axis, s.sign);
                const int ia = off + s.axis;
                const uint32_t n_ax = ia == 0 ? g.X : (ia == 1 ? g.Y : g.Z);
                if (n_ax < 2) return fail("lgb_step: outlet needs at least 2 cells along its normal");
                p.abb_k = k;
                p.abb_axis = ia;
                p.abb_sign = s.sign;
                p.abb_plane = s.sign > 0 ? n_ax - 1 : 0;
                p.abb_nb = s.sign > 0 ? n_ax - 2 : 1;
            }
        }
    }
    if (p.abb_k >= 0 && d->f_in == d->f_out)
        return fail("lgb_step: the anti-bounce-back outlet reads its neighbour plane and "
                    "needs distinct input and output fields");
    if (d->link_bits) {
        if (!masked) return fail("lgb_step: bounce-back links need the flag field");
        if (d->pattern != LGB_PULL && d->pattern != LGB_STREAM_ONLY && d->pattern != LGB_LOCAL)
            return fail("lgb_step: bounce-back links are applied by pulling streams "
                        "(LGB_PULL, LGB_STREAM_ONLY) and ignored by LGB_LOCAL; pattern %d",
                        d->pattern);
        p.links = d->link_bits;
        if (d->link_val) {
            if (!d->link_base || !d->link_pairs || !d->link_d || d->n_links <= 0 ||
                d->n_links > 0xffffffffLL)
                return fail("lgb_step: interpolated links need link_base, link_pairs, link_d "
                            "and 1..2^32-1 links (got %lld)", (long long)d->n_links);
            p.link_base = d->link_base;
            p.link_val = d->link_val;
        }
    } else if (d->force_links || d->force_out || d->link_val) {
        return fail("lgb_step: force_links / force_out / link_val without link_bits");
    }
    if (d->force_out && (d->n_force_links < 0 || (d->n_force_links > 0 && !d->force_links)))
        return fail("lgb_step: %lld force links at %p", (long long)d->n_force_links,
                    (const void *)d->force_links);
    if (d->force_out && !d->force_scratch)
        return fail("lgb_step: force_out needs force_scratch");
    if (d->force_out && d->n_force_links > 0xffffffffLL * LGB_LINK_FORCE_BLOCK)
        return fail("lgb_step: %lld force links", (long long)d->n_force_links);
    const bool streams = d->pattern == LGB_PULL || d->pattern == LGB_STREAM_ONLY;
    if (p.link_val && streams) {
        // the interpolated values come from f_in before the step reads them
        cudaError_t el = launch_link_values(d->stencil, d->storage, d->f_in, g, d->link_pairs,
                                            d->link_d, d->n_links, d->link_val,
                                            static_cast<cudaStream_t>(stream));
        if (el != cudaSuccess) return cuda_fail(el, "lgb_step: link value launch failed");
    }
    // the kernel variant: BGK with a force is its own collision kind; the
    // patterns without a collision (stream only, AA unpack) run as such
    // whatever the descriptor's collision
    const bool no_coll = d->pattern == LGB_STREAM_ONLY || d->pattern == LGB_AA_UNPACK;
    const int coll = no_coll ? LGB_NO_COLLISION
                     : (d->collision == LGB_BGK && d->force != LGB_FORCE_NONE ? lgb::LGB_BGK_FORCED
                                                                              : d->collision);
    const bool vec2 = !(d->options & LGB_OPT_ONE_CELL) &&
                      use_vec2(d->storage, coll, d->pattern, masked, g.Z);
    cudaError_t e = vec2
                        ? dispatch_step_vec2(d->stencil, d->storage, coll, d->pattern, p,
                                             static_cast<cudaStream_t>(stream))
                        : dispatch_step(d->stencil, d->storage, coll, d->pattern, masked,
                                        p, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "lgb_step: launch failed");
    if (d->force_out && streams) {
        // f_in still holds the post-collision field the links bounced
        e = launch_link_force(d->stencil, d->storage, d->f_in, g.N, d->force_links,
                              d->n_force_links, d->link_val, d->n_links, d->force_out,
                              d->force_scratch, static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return cuda_fail(e, "lgb_step: link force launch failed");
    }
    return 0;
}

int lgb_moments(int32_t stencil, int32_t storage, const int32_t *res, const void *f,
                int32_t aa_pending, void *rho, void *u, void *stream) {
    Grid g;
    if (make_grid(stencil, res, &g)) return -1;
    if (!valid_storage(storage)) return fail("lgb_moments: unknown storage id %d", storage);
    if (!f || !rho || !u) return fail("lgb_moments: NULL pointer");
    cudaError_t e = moments_dispatch(stencil, storage, g, f, aa_pending, rho, u,
                                     static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "lgb_moments: launch failed");
    return 0;
}

int64_t lgb_reduce_scratch_bytes(void) {
    return (int64_t)kReduceBlocks * LGB_REDUCE_FIELDS * (int64_t)sizeof(double);
}

int lgb_reduce(int32_t stencil, int32_t storage, const int32_t *res, const void *f,
               int32_t aa_pending, const int32_t *lo, const int32_t *hi, const uint8_t *mask,
               double *out, void *scratch, void *stream) {
    Grid g;
    if (make_grid(stencil, res, &g)) return -1;
    if (!valid_storage(storage)) return fail("lgb_reduce: unknown storage id %d", storage);
    if (!f || !out || !scratch) return fail("lgb_reduce: NULL pointer");
    ReduceBox box;
    const uint32_t full[3] = {g.X, g.Y, g.Z};
    for (int i = 0; i < 3; ++i) { box.lo[i] = 0; box.hi[i] = full[i]; }
    const int off = 3 - g.d;
    for (int i = 0; i < g.d; ++i) {
        const int32_t l = lo ? lo[i] : 0, h = hi ? hi[i] : (int32_t)full[off + i];
        if (l < 0 || h > (int32_t)full[off + i] || l > h)
            return fail("lgb_reduce: box [%d, %d) invalid along dimension %d", l, h, i);
        box.lo[off + i] = (uint32_t)l;
        box.hi[off + i] = (uint32_t)h;
    }
    cudaError_t e = reduce_dispatch(stencil, storage, g, f, aa_pending, box, mask, out,
                                    static_cast<double *>(scratch), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "lgb_reduce: launch failed");
    return 0;
}

}  // extern "C"

// ----------------------------------------------------------------------------
// Allocation-free reduction: lgb_reduce with its partial-sum scratch in a
// file-scope device array instead of a caller-provided buffer. The array is
// part of this library's device image, so every GPU that loads the library
// holds it (LGB_REDUCE_STATIC_SCRATCH_BYTES) until the process exits.

static __device__ __align__(256) double g_reduce_scratch[LGB_REDUCE_STATIC_SCRATCH_BYTES / sizeof(double)];

// the reduction launches a fixed grid of kReduceBlocks blocks whatever the
// field size, so its scratch need is a build-time constant
static_assert((int64_t)kReduceBlocks * LGB_REDUCE_FIELDS * (int64_t)sizeof(double) <=
                  (int64_t)LGB_REDUCE_STATIC_SCRATCH_BYTES,
              "the reduction's partial sums do not fit the static scratch array");

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// device address of g_reduce_scratch on the current device, looked up once
// per device (the host-side name g_reduce_scratch is not a device address).
// The cached address belongs to the device's context at the time of the
// lookup: after cudaDeviceReset the process must not call
// lgb_reduce_static on that device again (the header says so)
int static_scratch_address(void **ptr) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "lgb_reduce_static: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail("lgb_reduce_static: device ordinal %d beyond the %d supported", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_reduce_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "lgb_reduce_static: cudaGetSymbolAddress");
        g_scratch_addr[dev] = p;
    }
    *ptr = g_scratch_addr[dev];
    return 0;
}

}  // namespace

extern "C" {

int lgb_reduce_static(int32_t stencil, int32_t storage, const int32_t *res, const void *f,
                      int32_t aa_pending, const int32_t *lo, const int32_t *hi,
                      const uint8_t *mask, double *out, void *stream) {
    Grid g;
    if (make_grid(stencil, res, &g)) return -1;
    if (!valid_storage(storage)) return fail("lgb_reduce_static: unknown storage id %d", storage);
    if (!f || !out) return fail("lgb_reduce_static: NULL pointer");
    // the partial sums this call writes (a fixed grid of kReduceBlocks
    // blocks whatever the field size; the static_assert above holds it to
    // the array at build time, this keeps the run-time refusal beside it)
    const int64_t need = lgb_reduce_scratch_bytes();
    if (need > (int64_t)LGB_REDUCE_STATIC_SCRATCH_BYTES)
        return fail("lgb_reduce_static: the reduction needs %lld bytes of scratch, the static "
                    "array holds %lld", (long long)need, (long long)LGB_REDUCE_STATIC_SCRATCH_BYTES);
    ReduceBox box;
    const uint32_t full[3] = {g.X, g.Y, g.Z};
    for (int i = 0; i < 3; ++i) { box.lo[i] = 0; box.hi[i] = full[i]; }
    const int off = 3 - g.d;
    for (int i = 0; i < g.d; ++i) {
        const int32_t l = lo ? lo[i] : 0, h = hi ? hi[i] : (int32_t)full[off + i];
        if (l < 0 || h > (int32_t)full[off + i] || l > h)
            return fail("lgb_reduce_static: box [%d, %d) invalid along dimension %d", l, h, i);
        box.lo[off + i] = (uint32_t)l;
        box.hi[off + i] = (uint32_t)h;
    }
    void *scratch = nullptr;
    if (static_scratch_address(&scratch)) return -1;
    // every partial row the final fold reads is written earlier in the same
    // call, so the array needs no clearing between calls
    cudaError_t e = reduce_dispatch(stencil, storage, g, f, aa_pending, box, mask, out,
                                    static_cast<double *>(scratch), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "lgb_reduce_static: launch failed");
    return 0;
}

int lgb_host_pointer(const void *host, void **device) {
    if (!host || !device) return fail("lgb_host_pointer: NULL pointer");
    void *d = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&d, const_cast<void *>(host), 0);
    if (e != cudaSuccess || !d) {
        cudaGetLastError();  // not sticky; leave no error behind for the next call
        return fail("lgb_host_pointer: not page-locked, mapped host memory (%s)",
                    cudaGetErrorString(e));
    }
    *device = d;
    return 0;
}

int lgb_convert(int32_t stencil, int32_t src_storage, const void *src, int32_t dst_storage,
                void *dst, int64_t n_cells, void *stream) {
    int dd, q;
    if (stencil_dq(stencil, &dd, &q)) return fail("lgb_convert: unknown stencil id %d", stencil);
    if (!valid_storage(src_storage) || !valid_storage(dst_storage))
        return fail("lgb_convert: unknown storage id");
    if (!src || !dst) return fail("lgb_convert: NULL pointer");
    if (n_cells < 0) return fail("lgb_convert: negative cell count");
    if (n_cells == 0) return 0;
    cudaError_t e = convert_dispatch(stencil, src_storage, src, dst_storage, dst, (uint64_t)n_cells,
                                     static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "lgb_convert: launch failed");
    return 0;
}

}  // extern "C"
