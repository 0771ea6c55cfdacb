// Population storage formats. Loads return the population in the compute
// type R, stores take it back; the 16-bit formats hold f_q - w_q so that the
// small deviation from the rest equilibrium, not f_q itself, carries the 11
// (fp16) or 8 (bf16) mantissa bits.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

#include "lettuce_gb300.h"

namespace lgb {

template <int ST> struct Storage;

template <> struct Storage<LGB_F64> {
    using T = double;
    using R = double;
    static __device__ __forceinline__ R load(const T *p, double) { return __ldg(p); }
    static __device__ __forceinline__ R load_plain(const T *p, double) { return *p; }
    static __device__ __forceinline__ void store(T *p, R v, double) { *p = v; }
    static __device__ __forceinline__ void store_stream(T *p, R v, double) { __stcs(p, v); }
};

template <> struct Storage<LGB_F32> {
    using T = float;
    using R = float;
    static __device__ __forceinline__ R load(const T *p, double) { return __ldg(p); }
    static __device__ __forceinline__ R load_plain(const T *p, double) { return *p; }
    static __device__ __forceinline__ void store(T *p, R v, double) { *p = v; }
    static __device__ __forceinline__ void store_stream(T *p, R v, double) { __stcs(p, v); }
};

template <> struct Storage<LGB_F16_SHIFTED> {
    using T = __half;
    using R = float;
    static __device__ __forceinline__ R load(const T *p, double w) {
        return (float)w + __half2float(__ldg(p));
    }
    static __device__ __forceinline__ R load_plain(const T *p, double w) {
        return (float)w + __half2float(*p);
    }
    static __device__ __forceinline__ void store(T *p, R v, double w) {
        *p = __float2half_rn(v - (float)w);
    }
    static __device__ __forceinline__ void store_stream(T *p, R v, double w) {
        __stcs(reinterpret_cast<unsigned short *>(p),
               __half_as_ushort(__float2half_rn(v - (float)w)));
    }
    // the stored deviation h = f - w itself
    static __device__ __forceinline__ R load_h(const T *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void store_h(T *p, R h) { *p = __float2half_rn(h); }
};

template <> struct Storage<LGB_BF16_SHIFTED> {
    using T = __nv_bfloat16;
    using R = float;
    static __device__ __forceinline__ R load(const T *p, double w) {
        return (float)w + __bfloat162float(__ldg(p));
    }
    static __device__ __forceinline__ R load_plain(const T *p, double w) {
        return (float)w + __bfloat162float(*p);
    }
    static __device__ __forceinline__ void store(T *p, R v, double w) {
        *p = __float2bfloat16_rn(v - (float)w);
    }
    static __device__ __forceinline__ void store_stream(T *p, R v, double w) {
        __stcs(reinterpret_cast<unsigned short *>(p),
               __bfloat16_as_ushort(__float2bfloat16_rn(v - (float)w)));
    }
    static __device__ __forceinline__ R load_h(const T *p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ void store_h(T *p, R h) { *p = __float2bfloat16_rn(h); }
};

template <int ST> __host__ __device__ constexpr bool is_shifted() {
    return ST == LGB_F16_SHIFTED || ST == LGB_BF16_SHIFTED;
}

inline int storage_bytes(int st) {
    return st == LGB_F64 ? 8 : (st == LGB_F32 ? 4 : 2);
}

}  // namespace lgb
