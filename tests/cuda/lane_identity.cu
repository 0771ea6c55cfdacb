// Test program (built by tests/test_gpu_lane_identity.py): the shifted-space
// collision on one cell per thread (Lane1) and on two cells per thread with
// packed f32x2 arithmetic (Lane2) must agree bit for bit on random inputs.
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

#include "lgb_shifted.cuh"

using namespace lgb;

template <class S, int COLL>
__global__ void compare(const float *in, int pairs, CollideParams cp, unsigned long long *bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    float a[S::Q], b[S::Q];
    float2 v[S::Q];
    for (int q = 0; q < S::Q; ++q) {
        a[q] = in[(2 * i) * S::Q + q];
        b[q] = in[(2 * i + 1) * S::Q + q];
        v[q] = make_float2(a[q], b[q]);
    }
    collide_shifted<S, Lane1, COLL>(a, cp);
    collide_shifted<S, Lane1, COLL>(b, cp);
    collide_shifted<S, Lane2, COLL>(v, cp);
    for (int q = 0; q < S::Q; ++q)
        if (__float_as_uint(a[q]) != __float_as_uint(v[q].x) ||
            __float_as_uint(b[q]) != __float_as_uint(v[q].y))
            atomicAdd(bad, 1ull);
}

template <class S>
unsigned long long run(int coll, double tau, double tau_minus, int pairs, unsigned seed) {
    const int n = 2 * pairs;
    float *h = (float *)malloc(sizeof(float) * n * S::Q);
    srand(seed);
    for (int i = 0; i < n; ++i) {
        float u[3];
        for (int d = 0; d < 3; ++d) u[d] = 0.08f * ((float)rand() / RAND_MAX - 0.5f);
        const float drho = 0.02f * ((float)rand() / RAND_MAX - 0.5f);
        for (int q = 0; q < S::Q; ++q) {
            float eu = 0.f;
            for (int d = 0; d < S::D; ++d) eu += S::e(q, d) * u[d];
            const float w = (float)S::w(q);
            h[i * S::Q + q] = w * (drho + 3.f * eu + 4.5f * eu * eu) +
                              2e-4f * ((float)rand() / RAND_MAX - 0.5f);
        }
    }
    float *d;
    unsigned long long *bad;
    cudaMalloc(&d, sizeof(float) * n * S::Q);
    cudaMalloc(&bad, sizeof(unsigned long long));
    cudaMemset(bad, 0, sizeof(unsigned long long));
    cudaMemcpy(d, h, sizeof(float) * n * S::Q, cudaMemcpyHostToDevice);
    CollideParams cp;
    cp.omega = 1.0 / tau;
    cp.inv_2tp = 1.0 / (2.0 * tau);
    cp.inv_2tm = 1.0 / (2.0 * tau_minus);
    cp.beta = 1.0 / (2.0 * tau);
    set_float_rates(cp);
    const int blocks = (pairs + 255) / 256;
    if (coll == LGB_BGK) compare<S, LGB_BGK><<<blocks, 256>>>(d, pairs, cp, bad);
    else compare<S, LGB_TRT><<<blocks, 256>>>(d, pairs, cp, bad);
    unsigned long long hb = ~0ull;
    cudaMemcpy(&hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    if (cudaGetLastError() != cudaSuccess) hb = ~0ull;
    cudaFree(d);
    cudaFree(bad);
    free(h);
    return hb;
}

int main() {
    const int pairs = 1 << 20;
    unsigned long long total = 0;
    const double taus[2] = {0.5012, 0.93};
    for (int t = 0; t < 2; ++t) {
        for (int coll : {LGB_BGK, LGB_TRT}) {
            unsigned long long r2 = run<Stencil<LGB_D2Q9>>(coll, taus[t], 0.8, pairs, 1 + t);
            unsigned long long r19 = run<Stencil<LGB_D3Q19>>(coll, taus[t], 0.8, pairs, 3 + t);
            unsigned long long r27 = run<Stencil<LGB_D3Q27>>(coll, taus[t], 0.8, pairs, 5 + t);
            printf("tau %.4f collision %d: mismatches D2Q9 %llu D3Q19 %llu D3Q27 %llu\n", taus[t],
                   coll, r2, r19, r27);
            total += r2 + r19 + r27;
        }
    }
    printf("total mismatches %llu\n", total);
    return total == 0 ? 0 : 1;
}
