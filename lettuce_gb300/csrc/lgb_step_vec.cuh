// Two cells per thread for the shifted 16-bit population formats on grids
// without boundaries: every population of a cell pair is one 32-bit word
// (a half2 / bfloat162) of the row, so loads and stores are full-width and
// coalesced. A shift of the pair by one cell along the contiguous axis (the
// z component of e_q) straddles two words: both aligned words are loaded
// and one byte permute extracts the shifted pair (row ends wrap
// periodically). The collision runs on both cells at once with the packed
// f32x2 instructions (lgb_shifted.cuh), bit-identical to the one-cell path.
//
// Patterns: PULL, PUSH, LOCAL, AA_EVEN, AA_ODD. PUSH and AA_ODD store a
// shifted pair as two 16-bit halves (or, with LGB_VEC2_HALF_STORES 0,
// through a lane shuffle as whole words, halves only at row ends and warp
// edges); each half is written by exactly one thread.
#pragma once

#include "lgb_shifted.cuh"
#include "lgb_step.cuh"

namespace lgb {

template <int ST> struct Pack16;
template <> struct Pack16<LGB_F16_SHIFTED> {
    static __device__ __forceinline__ float2 decode(uint32_t w) {
        __half2 h = *reinterpret_cast<__half2 *>(&w);
        return __half22float2(h);
    }
    static __device__ __forceinline__ uint32_t encode(float2 v) {
        __half2 h = __float22half2_rn(v);
        return *reinterpret_cast<uint32_t *>(&h);
    }
};
template <> struct Pack16<LGB_BF16_SHIFTED> {
    static __device__ __forceinline__ float2 decode(uint32_t w) {
        __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&w);
        return __bfloat1622float2(h);
    }
    static __device__ __forceinline__ uint32_t encode(float2 v) {
        __nv_bfloat162 h = __float22bfloat162_rn(v);
        return *reinterpret_cast<uint32_t *>(&h);
    }
};

// PUSH / AA_ODD stores of a shifted pair: 16-bit halves at the shifted
// cells (1) or whole words composed through lane shuffles, with halves only
// at row ends and warp edges (0). Every half-word is written by the thread
// whose cell reads it in the same launch (for AA_ODD, cell x reads and
// writes slot q at x + e_q), so either form is race-free in place.
// Measured on D3Q19 fp16 256^3, AA pair: halves 73.8k MLUPS, shuffled
// words 72.8k (the shuffles, byte permutes and edge tests cost more issue
// slots than the second store saves).
#ifndef LGB_VEC2_HALF_STORES
#define LGB_VEC2_HALF_STORES 1
#endif

// the pair (z0 + dz, z0 + 1 + dz) of a row, dz in {-1, 0, 1}, from the
// aligned words at pair index tz and its periodic neighbours
__device__ __forceinline__ uint32_t load_pair(const uint32_t *__restrict__ row, uint32_t tz,
                                              uint32_t tzm, uint32_t tzp, int dz) {
    if (dz == 0) return __ldg(row + tz);
    if (dz < 0) return __byte_perm(__ldg(row + tzm), __ldg(row + tz), 0x5432);
    return __byte_perm(__ldg(row + tz), __ldg(row + tzp), 0x5432);
}

// the step of the cell pair tz (cells 2 tz, 2 tz + 1) of row (x, y) of the
// grid p. For PUSH and AA_ODD, pair t = row Z/2 + tz must be held by lane
// t mod 32 of a warp whose active lanes are `lanes`. INTERIOR: the row's x
// and y neighbours need no periodic wrap, so a neighbour row is the row
// plus a fixed offset (the wrap along z is handled either way).
template <int SID, int ST, int COLL, int PAT, bool INTERIOR>
__device__ __forceinline__ void step_pair_body(const StepParams &p, const uint32_t tz,
                                               const uint32_t x, const uint32_t y,
                                               const unsigned lanes) {
    using S = Stencil<SID>;
    using P = Pack16<ST>;
    const uint32_t Zh = p.Z >> 1;
    const uint32_t Nh = p.N >> 1;
    const uint32_t row = x * p.Y + y;
    const uint32_t tzm = tz == 0 ? Zh - 1 : tz - 1, tzp = tz + 1 == Zh ? 0 : tz + 1;
    const uint32_t *__restrict__ fin = static_cast<const uint32_t *>(p.f_in);
    auto row_of = [&](int dx, int dy) -> uint32_t {
        if constexpr (INTERIOR) {
            return row * Zh + (uint32_t)dx * (p.Y * Zh) + (uint32_t)dy * Zh;
        } else {
            const uint32_t xm = x == 0 ? p.X - 1 : x - 1, xp = x + 1 == p.X ? 0 : x + 1;
            const uint32_t ym = y == 0 ? p.Y - 1 : y - 1, yp = y + 1 == p.Y ? 0 : y + 1;
            const uint32_t a = dx == 0 ? x : (dx > 0 ? xp : xm);
            const uint32_t b = dy == 0 ? y : (dy > 0 ? yp : ym);
            return (a * p.Y + b) * Zh;
        }
    };

    float2 h[S::Q];
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        uint32_t w;
        if constexpr (PAT == LGB_PULL || PAT == LGB_AA_ODD) {
            const int slot = PAT == LGB_AA_ODD ? S::opp(q) : q;
            const uint32_t *r = fin + (size_t)slot * Nh + row_of(-ix<S>(q), -iy<S>(q));
            w = load_pair(r, tz, tzm, tzp, -iz<S>(q));
        } else {
            w = __ldg(fin + (size_t)q * Nh + row * Zh + tz);
        }
        h[q] = P::decode(w);
    }

    collide_shifted<S, Lane2, COLL>(h, p.cp);

    if (p.status) {
        float2 r = h[0];
#pragma unroll
        for (int q = 1; q < S::Q; ++q) r = Lane2::add(r, h[q]);
        if (!isfinite(r.x) || !isfinite(r.y)) atomicOr(p.status, 1u);
    }

    uint32_t *fout = static_cast<uint32_t *>(p.f_out);
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        const uint32_t w = P::encode(h[q]);
        if constexpr (PAT == LGB_PULL || PAT == LGB_LOCAL) {
            fout[(size_t)q * Nh + row * Zh + tz] = w;
        } else if constexpr (PAT == LGB_AA_EVEN) {
            fout[(size_t)S::opp(q) * Nh + row * Zh + tz] = w;
        } else {  // PUSH, AA_ODD: to (x, y, z) + e_q, slot q
            uint32_t *r = fout + (size_t)q * Nh + row_of(ix<S>(q), iy<S>(q));
            const int dz = iz<S>(q);
            if (dz == 0) {
                r[tz] = w;
            } else if constexpr (LGB_VEC2_HALF_STORES) {
                // each cell's value stored as its own 16-bit half at the
                // shifted cell (the two halves of a destination word come
                // from neighbouring lanes and meet in L2)
                unsigned short *r16 = reinterpret_cast<unsigned short *>(r);
                const uint32_t lo_dst = dz > 0 ? 2 * tz + 1 : (tz == 0 ? p.Z - 1 : 2 * tz - 1);
                const uint32_t hi_dst = dz > 0 ? (tz + 1 == Zh ? 0 : 2 * tz + 2) : 2 * tz;
                r16[lo_dst] = (unsigned short)(w & 0xffffu);
                r16[hi_dst] = (unsigned short)(w >> 16);
            } else {
                // the shifted pair straddles two words. A word whose two
                // halves come from pairs held by neighbouring lanes of one
                // row is composed by a shuffle and stored whole; at a row end
                // or a warp edge each half is stored alone by the lane that
                // holds its value (every half is written exactly once)
                unsigned short *r16 = reinterpret_cast<unsigned short *>(r);
                const uint32_t lane = threadIdx.x & 31u;
                if (dz > 0) {
                    // word tz = (cell 2tz - 1, cell 2tz) after the shift
                    const uint32_t prev = __shfl_up_sync(lanes, w, 1);
                    if (lane > 0 && tz > 0) r[tz] = __byte_perm(prev, w, 0x5432);
                    else r16[2 * tz + 1] = (unsigned short)(w & 0xffffu);
                    if (lane == 31 || tz + 1 == Zh)
                        r16[tz + 1 == Zh ? 0 : 2 * tz + 2] = (unsigned short)(w >> 16);
                } else {
                    // word tz = (cell 2tz + 1, cell 2tz + 2) after the shift
                    const uint32_t next = __shfl_down_sync(lanes, w, 1);
                    if (lane < 31 && tz + 1 < Zh) r[tz] = __byte_perm(w, next, 0x5432);
                    else r16[2 * tz] = (unsigned short)(w >> 16);
                    if (lane == 0 || tz == 0)
                        r16[tz == 0 ? p.Z - 1 : 2 * tz - 1] = (unsigned short)(w & 0xffffu);
                }
            }
        }
    }
}

// Interior rows (no wrap along x or y) take the fixed-offset form; the
// split is uniform over a warp whose pairs lie in one row. The shuffled
// scatter stores (LGB_VEC2_HALF_STORES 0) need every lane of `lanes` in one
// branch and keep the single form.
#ifndef LGB_VEC2_INTERIOR
#define LGB_VEC2_INTERIOR 1
#endif
template <int SID, int ST, int COLL, int PAT>
__device__ __forceinline__ void step_pair_at(const StepParams &p, const uint32_t tz,
                                             const uint32_t x, const uint32_t y,
                                             const unsigned lanes = 0xffffffffu) {
    using S = Stencil<SID>;
    constexpr bool NBR = PAT == LGB_PULL || PAT == LGB_PUSH || PAT == LGB_AA_ODD;
    constexpr bool SPLIT =
        LGB_VEC2_INTERIOR && NBR && (LGB_VEC2_HALF_STORES || PAT == LGB_PULL);
    if constexpr (SPLIT) {
        const bool interior = (S::D < 3 || (x > 0 && x + 1 < p.X)) &&
                              (S::D < 2 || (y > 0 && y + 1 < p.Y));
        if (interior) {
            step_pair_body<SID, ST, COLL, PAT, true>(p, tz, x, y, lanes);
            return;
        }
    }
    step_pair_body<SID, ST, COLL, PAT, false>(p, tz, x, y, lanes);
}

template <int SID, int ST, int COLL, int PAT>
__device__ __forceinline__ void step_pair(const StepParams &p, const uint32_t t,
                                          const unsigned lanes = 0xffffffffu) {
    const uint32_t row = p.divZ.div(t);
    const uint32_t x = p.divY.div(row);
    step_pair_at<SID, ST, COLL, PAT>(p, t - row * (p.Z >> 1), x, row - x * p.Y, lanes);
}

// four resident blocks per SM (64 registers): occupancy hides the load latency
// better than the registers the compiler would otherwise spend. D3Q27 (27
// population pairs) spills 100-400 bytes at 64 registers and gets its own
// bound.
#ifndef LGB_VEC2_D3Q27_MIN_BLOCKS
#define LGB_VEC2_D3Q27_MIN_BLOCKS 3
#endif
#ifndef LGB_VEC2_MIN_BLOCKS
#define LGB_VEC2_MIN_BLOCKS 4
#endif
// D2Q9 and D1Q3 (9 and 3 populations) need fewer registers: more blocks
// (measured on D2Q9 4096^2 fp16: 6 blocks 160.7k MLUPS, 5 blocks 154.1k, 4 blocks 141.1k)
#ifndef LGB_VEC2_2D_MIN_BLOCKS
#define LGB_VEC2_2D_MIN_BLOCKS 6
#endif
// the scattering patterns (PUSH, AA_ODD) of D3Q15 / D3Q19 keep the shuffled
// pair words of the stores live as well (32 bytes of spills at 64
// registers); 0 = the bound of their stencil. Measured on D3Q19 fp16 256^3,
// AA pair: 4 blocks per SM 72.8k MLUPS, 3 blocks (78 registers, no spills)
// 71.4k, 2 blocks 66.3k -- the spills cost less than the occupancy.
#ifndef LGB_VEC2_SCATTER_MIN_BLOCKS
#define LGB_VEC2_SCATTER_MIN_BLOCKS 0
#endif
template <int SID, int PAT>
constexpr int vec2_min_blocks() {
    return SID == LGB_D3Q27 ? LGB_VEC2_D3Q27_MIN_BLOCKS
           : (SID == LGB_D2Q9 || SID == LGB_D1Q3)
               ? LGB_VEC2_2D_MIN_BLOCKS
               : ((LGB_VEC2_SCATTER_MIN_BLOCKS > 0 && (PAT == LGB_PUSH || PAT == LGB_AA_ODD))
                      ? LGB_VEC2_SCATTER_MIN_BLOCKS
                      : LGB_VEC2_MIN_BLOCKS);
}
template <int SID, int ST, int COLL, int PAT>
__global__ void __launch_bounds__(256, (vec2_min_blocks<SID, PAT>()))
step_vec2_kernel(const StepParams p) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t Nh = p.N >> 1;
    if (t >= Nh) return;
    // lanes of this warp that hold a pair (blocks are whole warps)
    const uint32_t base = t & ~31u;
    const unsigned lanes = Nh - base >= 32u ? 0xffffffffu : (1u << (Nh - base)) - 1u;
    step_pair<SID, ST, COLL, PAT>(p, t, lanes);
}

template <int SID, int ST, int COLL, int PAT>
cudaError_t launch_step_vec2(const StepParams &p0, cudaStream_t stream) {
    StepParams p = p0;
    p.divZ = FastDiv::make(p.Z >> 1);
    const unsigned threads = 256;
    const unsigned blocks = (unsigned)(((p.N >> 1) + threads - 1) / threads);
    step_vec2_kernel<SID, ST, COLL, PAT><<<blocks, threads, 0, stream>>>(p);
    return cudaGetLastError();
}

template <int SID, int ST, int PAT>
cudaError_t dispatch_vec2_collision(int coll, const StepParams &p, cudaStream_t s) {
    switch (coll) {
    case LGB_NO_COLLISION: return launch_step_vec2<SID, ST, LGB_NO_COLLISION, PAT>(p, s);
    case LGB_BGK: return launch_step_vec2<SID, ST, LGB_BGK, PAT>(p, s);
    case LGB_TRT: return launch_step_vec2<SID, ST, LGB_TRT, PAT>(p, s);
    }
    return cudaErrorNotSupported;
}

template <int SID, int ST>
cudaError_t dispatch_vec2(int coll, int pat, const StepParams &p, cudaStream_t s) {
    switch (pat) {
    case LGB_PULL: return dispatch_vec2_collision<SID, ST, LGB_PULL>(coll, p, s);
    case LGB_PUSH: return dispatch_vec2_collision<SID, ST, LGB_PUSH>(coll, p, s);
    case LGB_LOCAL: return dispatch_vec2_collision<SID, ST, LGB_LOCAL>(coll, p, s);
    case LGB_AA_EVEN: return dispatch_vec2_collision<SID, ST, LGB_AA_EVEN>(coll, p, s);
    case LGB_AA_ODD: return dispatch_vec2_collision<SID, ST, LGB_AA_ODD>(coll, p, s);
    }
    return cudaErrorNotSupported;
}

#define LGB_DECLARE_VEC(name)                                                            \
    cudaError_t name##_s2(int, int, const StepParams &, cudaStream_t);                    \
    cudaError_t name##_s3(int, int, const StepParams &, cudaStream_t);
LGB_DECLARE_VEC(step_vec2_d1q3)
LGB_DECLARE_VEC(step_vec2_d2q9)
LGB_DECLARE_VEC(step_vec2_d3q15)
LGB_DECLARE_VEC(step_vec2_d3q19)
LGB_DECLARE_VEC(step_vec2_d3q27)
#undef LGB_DECLARE_VEC

}  // namespace lgb
