// Adjoint of the pull-pattern BGK step (lettuce PRE_STREAMING order):
//   f_{n+1}(x)_q = C(g(x))_q,  g(x)_q = f_n(x - e_q)_q,
//   C(g)_q = (1 - omega) g_q + omega feq_q(rho(g), u(g)).
// Given lambda_{n+1} = dL/df_{n+1}, the kernel forms at every cell x
//   mu_q = lambda_{n+1}(x)_q,
//   nu_p = (1 - omega) mu_p + omega (A + sum_d B_d (e_pd - u_d) / rho),
//   A   = sum_q mu_q feq_q / rho,
//   B_d = sum_q mu_q w_q rho (3 e_qd + 9 (e_q.u) e_qd - 3 u_d),
// (the chain rule through rho = sum g, u = sum e g / rho and the quadratic
// equilibrium of lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24)
// and scatters lambda_n(x - e_q)_q = nu_q: the transpose of the pull.
// Each (q, cell) of lambda_n is written by exactly one thread.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "lettuce_gb300.h"
#include "lgb_step.cuh"

namespace lgb {
int set_error(const char *msg);

template <int SID, int ST>
__global__ void __launch_bounds__(256) adjoint_bgk_kernel(const StepParams p, const void *lam_next_v,
                                                          void *lam_v) {
    using S = Stencil<SID>;
    using Sto = Storage<ST>;
    using R = typename Sto::R;
    using T = typename Sto::T;
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.N) return;
    const uint32_t row = p.divZ.div(n), z = n - row * p.Z;
    const uint32_t x = p.divY.div(row), y = row - x * p.Y;
    Nbr c;
    c.set(x, y, z, p);
    R g[S::Q];
    load_cell<S, Sto, LOAD_PULL, false>(p, static_cast<const T *>(p.f_in), c, n, 0u, g);
    const T *__restrict__ lam_next = static_cast<const T *>(lam_next_v);
    T *lam = static_cast<T *>(lam_v);
    const size_t N = p.N;
    R mu[S::Q];
#pragma unroll
    for (int q = 0; q < S::Q; ++q) mu[q] = (R)lam_next[(size_t)q * N + n];
    R rho, u[3];
    cell_moments<S>(g, rho, u);
    const R uu = dot_uu<S>(u);
    const R inv_rho = R(1) / rho;
    R A = R(0), B[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        R eu = R(0);
#pragma unroll
        for (int d = 0; d < S::D; ++d) eu += R(S::e(q, d)) * u[d];
        const R feq = feq_q<S>(q, rho, u, uu);
        A += mu[q] * feq * inv_rho;
        const R wr = R(S::w(q)) * rho * mu[q];
#pragma unroll
        for (int d = 0; d < S::D; ++d)
            B[d] += wr * (R(3) * R(S::e(q, d)) + R(9) * eu * R(S::e(q, d)) - R(3) * u[d]);
    }
    const R om = R(p.cp.omega);
    R Bu = R(0);
#pragma unroll
    for (int d = 0; d < S::D; ++d) Bu += B[d] * u[d];
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        R eB = R(0);
#pragma unroll
        for (int d = 0; d < S::D; ++d) eB += R(S::e(q, d)) * B[d];
        const R nu = (R(1) - om) * mu[q] + om * (A + (eB - Bu) * inv_rho);
        const uint32_t dst = c.at(-ix<S>(q), -iy<S>(q), -iz<S>(q), p);
        lam[(size_t)q * N + dst] = (T)nu;
    }
}

template <int SID>
cudaError_t launch_adjoint(int storage, const StepParams &p, const void *lam_next, void *lam,
                           cudaStream_t s) {
    const unsigned blocks = (p.N + 255) / 256;
    if (storage == LGB_F64)
        adjoint_bgk_kernel<SID, LGB_F64><<<blocks, 256, 0, s>>>(p, lam_next, lam);
    else if (storage == LGB_F32)
        adjoint_bgk_kernel<SID, LGB_F32><<<blocks, 256, 0, s>>>(p, lam_next, lam);
    else
        return cudaErrorNotSupported;
    return cudaGetLastError();
}

}  // namespace lgb

extern "C" int lgb_adjoint_step(int32_t stencil, int32_t storage, const int32_t *res, double tau,
                                const void *f_n, const void *lam_next, void *lam, void *stream) {
    char buf[256];
    int d = 0;
    switch (stencil) {
    case LGB_D1Q3: d = 1; break;
    case LGB_D2Q9: d = 2; break;
    case LGB_D3Q15: case LGB_D3Q19: case LGB_D3Q27: d = 3; break;
    default:
        snprintf(buf, sizeof(buf), "lgb_adjoint_step: unknown stencil id %d", stencil);
        return lgb::set_error(buf);
    }
    if (storage != LGB_F32 && storage != LGB_F64)
        return lgb::set_error("lgb_adjoint_step: the adjoint runs in float32 or float64 storage");
    if (!res || !f_n || !lam_next || !lam) return lgb::set_error("lgb_adjoint_step: NULL pointer");
    if (lam == lam_next || lam == f_n)
        return lgb::set_error("lgb_adjoint_step: the output must not alias an input");
    if (!(tau > 0.0)) return lgb::set_error("lgb_adjoint_step: tau must be positive");
    uint64_t r[3] = {1, 1, 1};
    for (int i = 0; i < d; ++i) {
        if (res[i] <= 0) return lgb::set_error("lgb_adjoint_step: resolution must be positive");
        r[3 - d + i] = (uint64_t)res[i];
    }
    if (r[0] * r[1] * r[2] >= (1ull << 32)) return lgb::set_error("lgb_adjoint_step: grid too large");
    lgb::StepParams p;
    memset(&p, 0, sizeof(p));
    p.f_in = f_n;
    p.X = (uint32_t)r[0]; p.Y = (uint32_t)r[1]; p.Z = (uint32_t)r[2];
    p.N = p.X * p.Y * p.Z;
    p.divZ = lgb::FastDiv::make(p.Z);
    p.divY = lgb::FastDiv::make(p.Y);
    p.cp.omega = 1.0 / tau;
    lgb::set_float_rates(p.cp);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaErrorInvalidValue;
    switch (stencil) {
    case LGB_D1Q3: e = lgb::launch_adjoint<LGB_D1Q3>(storage, p, lam_next, lam, s); break;
    case LGB_D2Q9: e = lgb::launch_adjoint<LGB_D2Q9>(storage, p, lam_next, lam, s); break;
    case LGB_D3Q15: e = lgb::launch_adjoint<LGB_D3Q15>(storage, p, lam_next, lam, s); break;
    case LGB_D3Q19: e = lgb::launch_adjoint<LGB_D3Q19>(storage, p, lam_next, lam, s); break;
    case LGB_D3Q27: e = lgb::launch_adjoint<LGB_D3Q27>(storage, p, lam_next, lam, s); break;
    }
    if (e != cudaSuccess) {
        snprintf(buf, sizeof(buf), "lgb_adjoint_step: launch failed: %s", cudaGetErrorString(e));
        return lgb::set_error(buf);
    }
    return 0;
}
