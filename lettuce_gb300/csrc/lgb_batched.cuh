// Batched step: many periodic domains of uneven sizes advanced by one
// launch. All domains' population fields live in one pool (domain b at
// element offset `offset`, layout [Q][N_b] as for a single grid); the host
// cuts every domain into tiles of whole rows (lgb_batch_plan) and the
// kernel's blocks walk the tile table with a grid stride (as many blocks as
// the SMs hold, or one block per tile), pulling from the periodic
// neighbours inside the tile's domain, with the domain's relaxation times.
// The float64 and float32 formats step one cell per thread. The 16-bit
// formats step two cells per thread, one 32-bit word per population pair
// (as lgb_step_vec.cuh does for a single grid): every row must be whole
// words -- an even row length, or an odd one stored with one pad element
// per row (pitch = length + 1) -- at an even offset; other domains are
// flagged and skipped.
#pragma once

#include "lgb_shifted.cuh"
#include "lgb_step.cuh"
#include "lgb_step_vec.cuh"

namespace lgb {

// the pulled pair (z0 + dz, z0 + 1 + dz) of a row of Zh words whose last
// word holds (cell Z - 1, pad): the periodic wrap skips the pad element
__device__ __forceinline__ uint32_t load_pair_padded(const uint32_t *__restrict__ row, uint32_t tz,
                                                     uint32_t Zh, int dz) {
    if (dz == 0) return __ldg(row + tz);
    if (dz < 0) {
        // (cell 2 tz - 1, cell 2 tz); left of cell 0 is cell Z - 1, the low
        // half of the last word
        if (tz == 0) return __byte_perm(__ldg(row + Zh - 1), __ldg(row), 0x5410);
        return __byte_perm(__ldg(row + tz - 1), __ldg(row + tz), 0x5432);
    }
    // (cell 2 tz + 1, cell 2 tz + 2); right of cell Z - 1 is cell 0 (the
    // last pair's second lane is the pad and takes cell 1)
    if (tz + 1 == Zh) return __ldg(row);
    return __byte_perm(__ldg(row + tz), __ldg(row + tz + 1), 0x5432);
}

struct BatchParams {
    const void *f_in;
    void *f_out;
    const lgb_batch_domain *domains;
    const lgb_batch_tile *tiles;
    int32_t n_domains;
    int32_t n_tiles;
    int64_t pool_elements;
    uint32_t *status;
    const float4 *rates;  // per domain, formed on the host (or null)
};

// The 16-bit pair loop keeps its tile's domain in shared memory and reads
// it there where it is used. Kernel parameters take no registers (they are
// read from the constant bank), a tile's grid, word offset and rates do:
// the D2Q9 fp16 TRT kernel took 62 registers with them held in registers,
// 50 with them in shared memory, which also fits the 48-register cap below
// without spills.

// a tile of a 16-bit domain as its pair loop reads it: three 16-byte
// groups, each read with one shared-memory load where it is used
struct alignas(16) TilePairs {
    uint32_t X, Y, Zh, Nh; // grid, words per row, words per population plane
    float f_omega, f_one_minus_omega, f_inv_2tp, f_inv_2tm;
    uint32_t word_lo, word_hi; // the domain's first 32-bit word in the pool
    uint32_t end;              // one past the tile's last pair (row Zh + word)
    uint32_t step_rows;        // blockDim / Zh: whole rows a thread advances
    uint32_t begin;            // the tile's first pair
    uint32_t kind;             // 0: skip the tile, 1: even rows, 2: padded odd rows
    uint32_t unused[2];
};

__device__ __forceinline__ uint4 lds_u4(const void *ptr) {
    uint4 v;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(ptr);
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
    return v;
}

// the pull step of the pairs t2, t2 + blockDim, ... below ts.end of a tile
// (pair index = row Zh + word), the tile's values read from shared memory in
// 16-byte groups where they are used; PADDED: the last word of a row holds
// (cell Z - 1, pad), the pad lane is left out of the status check. The next
// pair lies blockDim pairs on: ts.step_rows whole rows plus blockDim mod Zh
// words (no division, no per-row loop).
template <int SID, int ST, int COLL, bool PADDED>
__device__ __forceinline__ void tile_pairs_pull_vec(const BatchParams &p, const TilePairs &ts,
                                                    uint32_t t2) {
    using S = Stencil<SID>;
    using P = Pack16<ST>;
    const void *g_grid = &ts.X, *g_rates = &ts.f_omega, *g_tile = &ts.word_lo;
    // FLAT: a one- or two-dimensional grid (X = 1): the row is y, and no
    // pair of the tile lies past the last row
    constexpr bool FLAT = S::D < 3;
    uint32_t tz, x = 0, y;
    {
        const uint4 gr = lds_u4(g_grid);
        const uint32_t row = t2 / gr.z;
        tz = t2 - row * gr.z;
        if constexpr (FLAT) {
            y = row;
        } else {
            x = row / gr.y;
            y = row - x * gr.y;
        }
    }
    while (true) {
        float2 h[S::Q];
        {
            const uint4 gr = lds_u4(g_grid), tl = lds_u4(g_tile);
            const uint32_t X = gr.x, Y = gr.y, Zh = gr.z, Nh = gr.w;
            const uint32_t *__restrict__ fin = static_cast<const uint32_t *>(p.f_in) +
                                               (((uint64_t)tl.y << 32) | tl.x);
            const uint32_t xm = x == 0 ? X - 1 : x - 1, xp = x + 1 == X ? 0 : x + 1;
            const uint32_t ym = y == 0 ? Y - 1 : y - 1, yp = y + 1 == Y ? 0 : y + 1;
            const uint32_t tzm = tz == 0 ? Zh - 1 : tz - 1, tzp = tz + 1 == Zh ? 0 : tz + 1;
#pragma unroll
            for (int q = 0; q < S::Q; ++q) {
                const int dx = -ix<S>(q), dy = -iy<S>(q);
                const uint32_t a = dx == 0 ? x : (dx > 0 ? xp : xm);
                const uint32_t b = dy == 0 ? y : (dy > 0 ? yp : ym);
                const uint32_t *r = fin + (size_t)q * Nh + ((FLAT ? 0u : a * Y) + b) * Zh;
                uint32_t w;
                if constexpr (PADDED) w = load_pair_padded(r, tz, Zh, -iz<S>(q));
                else w = load_pair(r, tz, tzm, tzp, -iz<S>(q));
                h[q] = P::decode(w);
            }
        }
        {
            const uint4 rt = lds_u4(g_rates);
            CollideParams cp;
            cp.f_omega = __uint_as_float(rt.x);
            cp.f_one_minus_omega = __uint_as_float(rt.y);
            cp.f_inv_2tp = __uint_as_float(rt.z);
            cp.f_inv_2tm = __uint_as_float(rt.w);
            collide_shifted<S, Lane2, COLL>(h, cp);
        }
        const uint4 gr = lds_u4(g_grid), tl = lds_u4(g_tile);
        if (p.status) {
            float2 r = h[0];
#pragma unroll
            for (int q = 1; q < S::Q; ++q) r = Lane2::add(r, h[q]);
            if (!isfinite(r.x) || ((!PADDED || tz + 1 < gr.z) && !isfinite(r.y)))
                atomicOr(p.status, 1u);
        }
        {
            uint32_t *fout = static_cast<uint32_t *>(p.f_out) + (((uint64_t)tl.y << 32) | tl.x) +
                             ((FLAT ? 0u : x * gr.y) + y) * gr.z + tz;
#pragma unroll
            for (int q = 0; q < S::Q; ++q) fout[(size_t)q * gr.w] = P::encode(h[q]);
        }
        t2 += blockDim.x;
        if (t2 >= tl.z) break;
        tz += blockDim.x - tl.w * gr.z;
        y += tl.w;
        if (tz >= gr.z) { tz -= gr.z; ++y; }
        if constexpr (!FLAT) {
            while (y >= gr.y) { y -= gr.y; ++x; }
        }
    }
}

// One thread reads tile t and its domain, checks them as the per-thread
// path below does, and fills the block's TilePairs (kind 0 and status bit 1
// for a tile it refuses). The 16-bit pair loop needs nothing else of them.
template <int SID>
__device__ __forceinline__ void setup_tile_pairs(const BatchParams &p, const int t, TilePairs &ts) {
    using S = Stencil<SID>;
    ts.kind = 0;
    const lgb_batch_tile tile = p.tiles[t];
    if (tile.domain < 0 || tile.domain >= p.n_domains) {
        if (p.status) atomicOr(p.status, 2u);
        return;
    }
    const lgb_batch_domain dom = p.domains[tile.domain];
    const int d = S::D;
    uint32_t r[3] = {1, 1, 1};
    bool ok = true;
    for (int i = 0; i < d; ++i) {
        ok = ok && dom.res[i] > 0;
        r[3 - d + i] = (uint32_t)dom.res[i];
    }
    const uint32_t pitch = dom.pitch == 0 ? r[2] : (uint32_t)dom.pitch;
    const bool padded = pitch != r[2];
    ok = ok && dom.pitch >= 0 &&
         (!padded || ((r[2] & 1u) && pitch == r[2] + 1 && (dom.offset & 1) == 0));
    const uint64_t n_alloc = (uint64_t)r[0] * r[1] * pitch;
    ok = ok && n_alloc < (1ull << 32) && dom.offset >= 0 &&
         (uint64_t)dom.offset + (uint64_t)S::Q * n_alloc <= (uint64_t)p.pool_elements &&
         tile.row_begin >= 0 && tile.row_begin <= tile.row_end &&
         (uint64_t)tile.row_end <= (uint64_t)r[0] * r[1] && dom.tau > 0.0;
    // rows of whole 32-bit words: padded odd rows, or even rows at an even offset
    ok = ok && (padded || ((r[2] & 1u) == 0 && (dom.offset & 1) == 0));
    if (!ok) {
        if (p.status) atomicOr(p.status, 2u);
        return;
    }
    CollideParams c;
    if (p.rates) {
        const float4 fr = p.rates[tile.domain];
        c.f_omega = fr.x;
        c.f_one_minus_omega = fr.y;
        c.f_inv_2tp = fr.z;
        c.f_inv_2tm = fr.w;
    } else {
        c.omega = 1.0 / dom.tau;
        c.inv_2tp = 1.0 / (2.0 * dom.tau);
        c.inv_2tm = 1.0 / (2.0 * dom.tau_minus);
        set_float_rates(c);
    }
    ts.f_omega = c.f_omega;
    ts.f_one_minus_omega = c.f_one_minus_omega;
    ts.f_inv_2tp = c.f_inv_2tp;
    ts.f_inv_2tm = c.f_inv_2tm;
    const uint64_t word_offset = (uint64_t)dom.offset >> 1;
    const uint32_t Zh = pitch >> 1;
    ts.word_lo = (uint32_t)word_offset;
    ts.word_hi = (uint32_t)(word_offset >> 32);
    ts.X = r[0];
    ts.Y = r[1];
    ts.Zh = Zh;
    ts.Nh = (uint32_t)(n_alloc >> 1);
    ts.end = (uint32_t)tile.row_end * Zh;
    ts.step_rows = blockDim.x / Zh;
    ts.begin = (uint32_t)tile.row_begin * Zh;
    ts.kind = padded ? 2u : 1u;
}

// the one-cell pull step over tile t (float64 and float32 formats): every
// thread reads and checks the tile and its domain, one thread forms the
// rates for the block
template <int SID, int ST, int COLL>
__device__ __forceinline__ void batched_tile_cells(const BatchParams &p, const int t,
                                                   double (&s_rates)[3], float (&s_frates)[4]) {
    using S = Stencil<SID>;
    using Sto = Storage<ST>;
    using R = typename Sto::R;
    using T = typename Sto::T;
    static_assert(!is_shifted<ST>(), "the 16-bit formats take the pair loop");
    constexpr bool HSPACE = false;
    const T *__restrict__ pool_in = static_cast<const T *>(p.f_in);
    T *pool_out = static_cast<T *>(p.f_out);
    {
        const lgb_batch_tile tile = p.tiles[t];
        if (tile.domain < 0 || tile.domain >= p.n_domains) {
            if (threadIdx.x == 0 && p.status) atomicOr(p.status, 2u);
            return;
        }
        const lgb_batch_domain dom = p.domains[tile.domain];
        // the domain as an internal (X, Y, Z) grid
        StepParams g;
        const int d = S::D;
        uint32_t r[3] = {1, 1, 1};
        bool ok = true;
        for (int i = 0; i < d; ++i) {
            ok = ok && dom.res[i] > 0;
            r[3 - d + i] = (uint32_t)dom.res[i];
        }
        g.X = r[0]; g.Y = r[1]; g.Z = r[2];
        const uint64_t n64 = (uint64_t)r[0] * r[1] * r[2];
        // row pitch: the row length, or (16-bit shifted formats, odd row
        // length) one more, a pad element per row
        const uint32_t pitch = dom.pitch == 0 ? r[2] : (uint32_t)dom.pitch;
        const bool padded = pitch != r[2];
        ok = ok && dom.pitch >= 0 &&
             (!padded || (HSPACE && (r[2] & 1u) && pitch == r[2] + 1 && (dom.offset & 1) == 0));
        const uint64_t n_alloc = (uint64_t)r[0] * r[1] * pitch;
        // the tile must lie inside its domain and the domain inside the pool
        ok = ok && n_alloc < (1ull << 32) && dom.offset >= 0 &&
             (uint64_t)dom.offset + (uint64_t)S::Q * n_alloc <= (uint64_t)p.pool_elements &&
             tile.row_begin >= 0 && tile.row_begin <= tile.row_end &&
             (uint64_t)tile.row_end <= (uint64_t)r[0] * r[1] && dom.tau > 0.0;
        if (!ok) {
            if (threadIdx.x == 0 && p.status) atomicOr(p.status, 2u);
            return;
        }
        g.N = (uint32_t)n64;
        // the domain's relaxation rates, three float64 divisions: one thread
        // forms them and the block reads them from shared memory (formed by
        // every thread they kept the float64 pipe busy for a fifth of the
        // launch). Every thread of the block walks the same tile, so the
        // branches above are uniform and every thread reaches both barriers.
        __syncthreads();  // the previous tile's rates have been read
        if (threadIdx.x == 0) {
            // the float32 rates the collisions of the float32 and 16-bit
            // formats use: from the host's table, or rounded here from the
            // float64 quotients (the same values); the float32 collision
            // takes its rates back from the doubles exactly
            CollideParams c;
            if (p.rates) {
                const float4 fr = p.rates[tile.domain];
                c.f_omega = fr.x;
                c.f_one_minus_omega = fr.y;
                c.f_inv_2tp = fr.z;
                c.f_inv_2tm = fr.w;
                s_rates[0] = (double)fr.x;
                s_rates[1] = (double)fr.z;
                s_rates[2] = (double)fr.w;
            } else {
                s_rates[0] = 1.0 / dom.tau;
                s_rates[1] = 1.0 / (2.0 * dom.tau);
                s_rates[2] = 1.0 / (2.0 * dom.tau_minus);
                c.omega = s_rates[0];
                c.inv_2tp = s_rates[1];
                c.inv_2tm = s_rates[2];
                set_float_rates(c);
            }
            s_frates[0] = c.f_omega;
            s_frates[1] = c.f_one_minus_omega;
            s_frates[2] = c.f_inv_2tp;
            s_frates[3] = c.f_inv_2tm;
        }
        __syncthreads();
        CollideParams cp;
        cp.omega = s_rates[0];
        cp.inv_2tp = s_rates[1];
        cp.inv_2tm = s_rates[2];
        cp.beta = s_rates[1];
        cp.f_omega = s_frates[0];
        cp.f_one_minus_omega = s_frates[1];
        cp.f_inv_2tp = s_frates[2];
        cp.f_inv_2tm = s_frates[3];
        const T *__restrict__ fin = pool_in + dom.offset;
        T *fout = pool_out + dom.offset;
        // a thread's cells advance by blockDim along the tile's rows: the
        // row and column are carried forward (one division per tile instead
        // of fast-division constants derived per tile)
        const uint32_t step = blockDim.x;
        const uint32_t end = (uint32_t)tile.row_end * g.Z;
        uint32_t n = (uint32_t)tile.row_begin * g.Z + threadIdx.x;
        if (n >= end) return;
        uint32_t row = n / g.Z, z = n - row * g.Z;
        uint32_t x = row / g.Y, y = row - x * g.Y;
        while (true) {
            Nbr c;
            c.set(x, y, z, g);
            R f[S::Q];
            load_cell<S, Sto, LOAD_PULL, false, HSPACE>(g, fin, c, n, 0u, f);
            if constexpr (HSPACE) {
                collide_shifted<S, Lane1, COLL>(f, cp);
            } else {
                R rr;
                collide<COLL, S>(f, cp, rr);
            }
            if (p.status) {
                R s = R(0);
#pragma unroll
                for (int q = 0; q < S::Q; ++q) s += f[q];
                if (!isfinite(s)) atomicOr(p.status, 1u);
            }
            const size_t N = g.N;
#pragma unroll
            for (int q = 0; q < S::Q; ++q) store_value<Sto, HSPACE>(fout + (size_t)q * N + n, f[q], S::w(q));
            n += step;
            if (n >= end) break;
            z += step;
            while (z >= g.Z) {
                z -= g.Z;
                if (++y == g.Y) { y = 0; ++x; }
            }
        }
    }
}

// the batched step (one launch over every tile of the batch)
template <int SID, int ST, int COLL>
__device__ __forceinline__ void batched_step_body(const BatchParams &p) {
    constexpr bool HSPACE = is_shifted<ST>() && shifted_collision<COLL>();
    __shared__ double s_rates[3];
    __shared__ float s_frates[4];
    __shared__ TilePairs s_pairs;
    for (int t = blockIdx.x; t < p.n_tiles; t += gridDim.x) {
        if constexpr (HSPACE) {
            // the 16-bit pair loop: one thread sets the tile up (the loop
            // bounds are uniform, so every thread reaches both barriers)
            if (t != (int)blockIdx.x) __syncthreads();  // the previous tile is read
            if (threadIdx.x == 0) setup_tile_pairs<SID>(p, t, s_pairs);
            __syncthreads();
            const uint4 bk = lds_u4(&s_pairs.begin);
            if (bk.y != 0) {
                const uint32_t t2 = bk.x + threadIdx.x;
                if (t2 < lds_u4(&s_pairs.word_lo).z) {
                    if (bk.y == 2u) tile_pairs_pull_vec<SID, ST, COLL, true>(p, s_pairs, t2);
                    else tile_pairs_pull_vec<SID, ST, COLL, false>(p, s_pairs, t2);
                }
            }
        } else {
            batched_tile_cells<SID, ST, COLL>(p, t, s_rates, s_frates);
        }
    }
}

// Registers. The D2Q9 / D1Q3 batches of the 16-bit formats are capped at
// LGB_BATCH_16BIT_2D_MAXREG, those of float32 at LGB_BATCH_F32_2D_MAXREG
// (10 and 12 resident 128-thread blocks per SM instead of 8, no spills);
// the other batches keep the compiler's choice. Measured on the 256
// config-4 domains, fp16 TRT, best launch shape of each: the pair loop with
// its tile in registers 132.9k MLUPS (62 registers); with its tile in shared
// memory 126.1k (50), capped at 48 140.0k (no spills), at 44 136.6k (20
// bytes of spills), at 40 134.8k (48 bytes); reading the tile's values as
// 16-byte loads with a division-free advance, capped at 48, 143.0k against
// 140.3k (at 44: 20 bytes of spills); with the domains' float32 rates
// formed on the host (no float64 quotient per tile) 145.4k, and with one
// thread setting each tile up for the block 146.7k, and with the
// two-dimensional grids' x dropped from the pair loop 148.1k, and with the
// approximate reciprocal of the density (lgb_shifted.cuh) 150.9k. With the
// next pair's words copied asynchronously (cp.async, 4 bytes each) into a
// two-stage shared-memory buffer while the current pair collides: 110.8k.
// Float32:
// 76.2k uncapped (64 registers), 84.4k at 40, 82.8k at 32 (20 bytes of
// spills); 85.0k with the host's rates.
#ifndef LGB_BATCH_16BIT_2D_MAXREG
#define LGB_BATCH_16BIT_2D_MAXREG 48
#endif
#ifndef LGB_BATCH_F32_2D_MAXREG
#define LGB_BATCH_F32_2D_MAXREG 40
#endif
template <int SID, int ST>
constexpr int batch_maxreg() {
    return (SID != LGB_D2Q9 && SID != LGB_D1Q3) ? 0
           : is_shifted<ST>()                    ? LGB_BATCH_16BIT_2D_MAXREG
           : ST == LGB_F32                       ? LGB_BATCH_F32_2D_MAXREG
                                                 : 0;
}

template <int SID, int ST, int COLL>
__global__ void __launch_bounds__(512) batched_step_kernel(const BatchParams p) {
    batched_step_body<SID, ST, COLL>(p);
}

template <int SID, int ST, int COLL>
__global__ void __maxnreg__((batch_maxreg<SID, ST>() > 0 ? batch_maxreg<SID, ST>() : 64))
batched_step_kernel_capped(const BatchParams p) {
    batched_step_body<SID, ST, COLL>(p);
}

template <int SID, int ST, int COLL>
void launch_batched_as(const BatchParams &p, int blocks, int threads, cudaStream_t s) {
    if constexpr (batch_maxreg<SID, ST>() > 0)
        batched_step_kernel_capped<SID, ST, COLL><<<blocks, threads, 0, s>>>(p);
    else
        batched_step_kernel<SID, ST, COLL><<<blocks, threads, 0, s>>>(p);
}

template <int SID, int ST>
cudaError_t launch_batched(int coll, const BatchParams &p, int blocks, int threads, cudaStream_t s) {
    switch (coll) {
    case LGB_NO_COLLISION: launch_batched_as<SID, ST, LGB_NO_COLLISION>(p, blocks, threads, s); break;
    case LGB_BGK: launch_batched_as<SID, ST, LGB_BGK>(p, blocks, threads, s); break;
    case LGB_TRT: launch_batched_as<SID, ST, LGB_TRT>(p, blocks, threads, s); break;
    default: return cudaErrorNotSupported;
    }
    return cudaGetLastError();
}

template <int SID>
cudaError_t dispatch_batched(int storage, int coll, const BatchParams &p, int blocks, int threads,
                             cudaStream_t s) {
    switch (storage) {
    case LGB_F64: return launch_batched<SID, LGB_F64>(coll, p, blocks, threads, s);
    case LGB_F32: return launch_batched<SID, LGB_F32>(coll, p, blocks, threads, s);
    case LGB_F16_SHIFTED: return launch_batched<SID, LGB_F16_SHIFTED>(coll, p, blocks, threads, s);
    case LGB_BF16_SHIFTED: return launch_batched<SID, LGB_BF16_SHIFTED>(coll, p, blocks, threads, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lgb
