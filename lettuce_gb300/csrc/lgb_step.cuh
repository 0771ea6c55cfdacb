// Generic fused lattice Boltzmann step: one thread per cell, populations in
// registers, every access pattern of the C ABI (pull / push / local / AA
// even / AA odd / stream only) and lettuce's masked substep sequence.
//
// Semantics reproduced (lettuce/_simulation.py):
//   * stream (:241-256): f[q](x) <- f[q](x - e_q), periodic wrap; where the
//     no-streaming mask of (q, x) is set the destination keeps its value.
//   * masked collide (:258-305): substeps k = 0..n-1 (pre-boundaries,
//     collision, post-boundaries); a cell runs the substep whose index its
//     no-collision mask holds. The anti-bounce-back outlet mutates its plane
//     in place whatever that index is (anti_bounce_back_outlet.py:71-91), at
//     its position in the sequence, reading the neighbour plane's velocity
//     as it stands after the substeps before it.
//   * PRE_STREAMING = stream then collide, POST_STREAMING = collide then
//     stream (:148-166).
#pragma once

#include <cuda_runtime.h>

#include "lgb_collide.cuh"
#include "lgb_shifted.cuh"
#include "lgb_storage.cuh"

namespace lgb {

struct FastDiv {
    uint32_t d, m, s;
    static FastDiv make(uint32_t d) {
        FastDiv f;
        f.d = d;
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;
        f.s = l;
        f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        if (s == 0) return n;
        const uint32_t t = __umulhi(m, n);
        return (t + ((n - t) >> 1)) >> (s - 1);
    }
};

struct SubParams {
    int32_t kind;
    int32_t pad;
    const void *rho;  // equilibrium BC density (compute type)
    const void *u;    // equilibrium BC velocity (compute type)
    int64_t rs[3];    // density strides, internal X, Y, Z
    int64_t us[4];    // velocity strides: component, internal X, Y, Z
    double param[2];  // partially saturated: tau, B
};

struct StepParams {
    const void *f_in;
    void *f_out;
    // MRT tables in host memory (read by the launch, not by the kernel)
    const double *mrt_host;
    int32_t mrt_eq;
    uint32_t X, Y, Z, N;
    FastDiv divZ, divY;
    CollideParams cp;
    const uint8_t *flags;
    const uint32_t *nsb;
    const uint32_t *links;       // bounce-back link bits, or null
    const uint32_t *link_base;   // interpolated links: first link of a cell
    const void *link_val;        // interpolated links: bounced values (R), or null
    int32_t has_nsm;
    int32_t push_guard;  // the flags carry LGB_FLAG_PUSH_GUARD
    int32_t n_sub;
    int32_t coll_idx;    // substep index of the collision
    // the anti-bounce-back outlet (at most one): its substep index (-1 for
    // none), internal axis of its normal (0=X, 1=Y, 2=Z), sign, plane and
    // neighbour-plane coordinates along that axis
    int32_t abb_k, abb_axis, abb_sign;
    uint32_t abb_plane, abb_nb;
    int32_t abb_kind;   // LGB_SUB_ANTI_BOUNCE_BACK or LGB_SUB_EQUILIBRIUM_OUTLET_P
    double abb_rho;     // pressure outlet density
    SubParams sub[LGB_MAX_SUBSTEPS];
    uint32_t *status;
};

// coordinates of a cell and of its periodic neighbours
struct Nbr {
    uint32_t x, y, z, xm, xp, ym, yp, zm, zp;
    __device__ __forceinline__ void set(uint32_t x_, uint32_t y_, uint32_t z_, const StepParams &p) {
        x = x_; y = y_; z = z_;
        xm = x == 0 ? p.X - 1 : x - 1; xp = x + 1 == p.X ? 0 : x + 1;
        ym = y == 0 ? p.Y - 1 : y - 1; yp = y + 1 == p.Y ? 0 : y + 1;
        zm = z == 0 ? p.Z - 1 : z - 1; zp = z + 1 == p.Z ? 0 : z + 1;
    }
    // cell index of (x, y, z) + (dx, dy, dz), each in {-1, 0, 1}
    __device__ __forceinline__ uint32_t at(int dx, int dy, int dz, const StepParams &p) const {
        const uint32_t a = dx == 0 ? x : (dx > 0 ? xp : xm);
        const uint32_t b = dy == 0 ? y : (dy > 0 ? yp : ym);
        const uint32_t c = dz == 0 ? z : (dz > 0 ? zp : zm);
        return (a * p.Y + b) * p.Z + c;
    }
};

enum LoadKind { LOAD_OWN, LOAD_PULL, LOAD_AA_ODD };

template <int PAT> struct PatternTraits;
template <> struct PatternTraits<LGB_PULL> { static constexpr int load = LOAD_PULL; };
template <> struct PatternTraits<LGB_STREAM_ONLY> { static constexpr int load = LOAD_PULL; };
template <> struct PatternTraits<LGB_PUSH> { static constexpr int load = LOAD_OWN; };
template <> struct PatternTraits<LGB_LOCAL> { static constexpr int load = LOAD_OWN; };
template <> struct PatternTraits<LGB_AA_EVEN> { static constexpr int load = LOAD_OWN; };
template <> struct PatternTraits<LGB_AA_ODD> { static constexpr int load = LOAD_AA_ODD; };
template <> struct PatternTraits<LGB_AA_UNPACK> { static constexpr int load = LOAD_AA_ODD; };

// populations of the cell `c` (index n) as the collide phase sees them
template <class S, class Sto, int LOAD, bool MASKED, bool RAW = false, bool LINKS = false>
__device__ __forceinline__ void load_cell(const StepParams &p, const typename Sto::T *__restrict__ fin,
                                          const Nbr &c, uint32_t n, uint32_t nsbits,
                                          typename Sto::R (&f)[S::Q], uint32_t lbits = 0) {
    const size_t N = p.N;
    // a pull with no-streaming bits keeps the cell's own value for those
    // populations, and a halfway bounce-back link takes the cell's own
    // opposite population; cells without either (nearly all) skip the
    // per-population test
    const bool keep_own = MASKED && LOAD == LOAD_PULL && (nsbits | (LINKS ? lbits : 0u)) != 0;
    using T = typename Sto::T;
    auto load_all = [&](const bool check) {
#pragma unroll
        for (int q = 0; q < S::Q; ++q) {
            uint32_t src = n;
            int slot = q;
            if (LOAD == LOAD_PULL || LOAD == LOAD_AA_ODD) {
                src = c.at(-ix<S>(q), -iy<S>(q), -iz<S>(q), p);
                if (LOAD == LOAD_AA_ODD) slot = S::opp(q);
            }
            const T *ptr = fin + (size_t)slot * N + src;
            if (LOAD == LOAD_PULL && check && q != 0) {
                // the bounce follows the stream (halfway_bounce_back_boundary.py:
                // 182-190 runs after ebb_simulation.py:76), so a link wins
                // over a no-streaming bit. A halfway link takes the cell's own
                // post-collision opp(q); an interpolated one the value the
                // link pass stored (same storage format)
                if (LINKS && ((lbits >> q) & 1u))
                    ptr = p.link_val ? static_cast<const T *>(p.link_val) + p.link_base[n] +
                                           __popc(lbits & ((1u << q) - 1u))
                                     : fin + (size_t)S::opp(q) * N + n;
                else if ((nsbits >> q) & 1u)
                    ptr = fin + (size_t)q * N + n;
            }
            if constexpr (RAW) f[q] = Sto::load_h(ptr);
            else f[q] = Sto::load(ptr, S::w(q));
        }
    };
    if (keep_own) load_all(true);
    else load_all(false);
}

// the substep with index `idx`, copied out of the parameter block by an
// unrolled select so no dynamic indexing of kernel parameters is needed
__device__ __forceinline__ SubParams select_sub(const StepParams &p, int idx) {
    SubParams r;
    r.kind = LGB_SUB_NONE;
    r.rho = nullptr;
    r.u = nullptr;
    r.param[0] = r.param[1] = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) r.rs[d] = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) r.us[d] = 0;
#pragma unroll
    for (int k = 0; k < LGB_MAX_SUBSTEPS; ++k) {
        if (k == idx && k < p.n_sub) {
            r.kind = p.sub[k].kind;
            r.rho = p.sub[k].rho;
            r.u = p.sub[k].u;
#pragma unroll
            for (int d = 0; d < 3; ++d) r.rs[d] = p.sub[k].rs[d];
#pragma unroll
            for (int d = 0; d < 4; ++d) r.us[d] = p.sub[k].us[d];
            r.param[0] = p.sub[k].param[0];
            r.param[1] = p.sub[k].param[1];
        }
    }
    return r;
}

// substep `sb` (collision, bounce-back, equilibrium BC or none) at one cell
template <class S, int COLL, bool WITH_COLLISION = true, class R, class TT>
__device__ __forceinline__ void apply_local_substep(const StepParams &p, const SubParams &sb,
                                                    const Nbr &c, R (&f)[S::Q], const TT &tab) {
    if (WITH_COLLISION && sb.kind == LGB_SUB_COLLISION) {
        R r;
        collide<COLL, S>(f, p.cp, r, tab);
    } else if (sb.kind == LGB_SUB_BOUNCE_BACK) {
        // bounce_back_boundary.py:17-18: f <- f[opposite]
#pragma unroll
        for (int q = 1; q < S::Q; ++q) {
            const int o = S::opp(q);
            if (q < o) { const R t = f[q]; f[q] = f[o]; f[o] = t; }
        }
    } else if (sb.kind == LGB_SUB_EQUILIBRIUM_PU) {
        // equilibrium_boundary_pu.py:79-84: f <- feq(rho(p), u)
        const R *rp = static_cast<const R *>(sb.rho);
        const R *up = static_cast<const R *>(sb.u);
        const R rho = rp[(int64_t)c.x * sb.rs[0] + (int64_t)c.y * sb.rs[1] + (int64_t)c.z * sb.rs[2]];
        const int64_t ub = (int64_t)c.x * sb.us[1] + (int64_t)c.y * sb.us[2] + (int64_t)c.z * sb.us[3];
        R u[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = d < S::D ? up[ub + d * sb.us[0]] : R(0);
        set_equilibrium<S>(f, rho, u);
    } else if (sb.kind == LGB_SUB_PARTIALLY_SATURATED) {
        // partially_saturated_boundary.py:24-41 (Noble & Torczynski 1998):
        // f - (1 - B)/tau (f - feq) + B ((f_opp - feq_opp) - (f - feq(rho, 0)))
        R rho, u[3];
        cell_moments<S>(f, rho, u);
        const R uu = dot_uu<S>(u);
        const R tau = R(sb.param[0]), B = R(sb.param[1]);
        const R a = (R(1) - B) / tau;
        R out[S::Q];
#pragma unroll
        for (int q = 0; q < S::Q; ++q) {
            const int o = S::opp(q);
            const R fe = feq_q<S>(q, rho, u, uu), fo = feq_q<S>(o, rho, u, uu);
            out[q] = f[q] - a * (f[q] - fe) + B * ((f[o] - fo) - (f[q] - R(S::w(q)) * rho));
        }
#pragma unroll
        for (int q = 0; q < S::Q; ++q) f[q] = out[q];
    }
}

__device__ __forceinline__ uint32_t coord_along(const Nbr &c, int axis) {
    return axis == 0 ? c.x : (axis == 1 ? c.y : c.z);
}

// the outlet-plane substep at a cell of the plane: anti-bounce-back
// (anti_bounce_back_outlet.py:71-91) or pressure outlet
// (equilibrium_outlet_p.py:61-71). The neighbour one cell inside is rebuilt
// as the collide phase sees it at substep abb_k (its populations after the
// substeps before abb_k).
template <class S, int COLL, int LOAD, bool MASKED, bool LINKS, class Sto, class TT>
__device__ __forceinline__ void apply_outlet(const StepParams &p, const typename Sto::T *__restrict__ fin,
                                             const Nbr &c, typename Sto::R (&f)[S::Q], const TT &tab) {
    using R = typename Sto::R;
    uint32_t xn = c.x, yn = c.y, zn = c.z;
    if (p.abb_axis == 0) xn = p.abb_nb; else if (p.abb_axis == 1) yn = p.abb_nb; else zn = p.abb_nb;
    Nbr cn;
    cn.set(xn, yn, zn, p);
    const uint32_t nn = (xn * p.Y + yn) * p.Z + zn;
    const uint8_t fl = p.flags[nn];
    const uint32_t nsb = ((fl & LGB_FLAG_NO_STREAM) && p.nsb) ? p.nsb[nn] : 0u;
    const uint32_t lb =
        (LINKS && LOAD == LOAD_PULL && (fl & LGB_FLAG_LINKS) && p.links) ? p.links[nn] : 0u;
    R g[S::Q];
    load_cell<S, Sto, LOAD, MASKED, false, LINKS>(p, fin, cn, nn, nsb, g, lb);
    const int idx = fl & LGB_FLAG_INDEX_MASK;
    if (idx < p.abb_k) apply_local_substep<S, COLL>(p, select_sub(p, idx), cn, g, tab);
    R rho, u[3], rn, un[3];
    cell_moments<S>(g, rn, un);
    if (p.abb_kind == LGB_SUB_EQUILIBRIUM_OUTLET_P) {
        // equilibrium_outlet_p.py:61-71: the plane takes the equilibrium of
        // the outlet density and the neighbour plane's velocity
        set_equilibrium<S>(f, R(p.abb_rho), un);
        return;
    }
    cell_moments<S>(f, rho, u);
    R uw[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) uw[d] = u[d] + R(0.5) * (u[d] - un[d]);
    const R uu = dot_uu<S>(uw);
#pragma unroll
    for (int q = 1; q < S::Q; ++q) {
        const int along = p.abb_axis == 0 ? ix<S>(q) : (p.abb_axis == 1 ? iy<S>(q) : iz<S>(q));
        if (along * p.abb_sign == 1) {
            R eu = R(0);
#pragma unroll
            for (int d = 0; d < S::D; ++d) eu += R(S::e(q, d)) * uw[d];
            // cs^-4 = 9, cs^-2 = 3
            f[S::opp(q)] = -f[q] + R(S::w(q)) * rho * (R(2) + eu * eu * R(9) - uu * R(3));
        }
    }
}

template <class Sto, bool RAW>
__device__ __forceinline__ void store_value(typename Sto::T *ptr, typename Sto::R v, double w) {
    if constexpr (RAW) Sto::store_h(ptr, v);
    else Sto::store(ptr, v, w);
}

// D3Q27 KBC in float32 with the pulling / collide-only patterns: the cell's 27
// populations go through a shared-memory stage (one column per thread,
// [Q][256], consecutive threads in consecutive banks) and the collision reads
// them back for each of its passes (moments, entropic sums, update) instead
// of holding them in registers across the passes. Same operations in the
// same order as the register form; the registers freed raise the resident
// blocks per SM.
#ifndef LGB_KBC_STAGE
#define LGB_KBC_STAGE 0
#endif
constexpr int kStageThreads = 256;
template <int SID, int ST, int COLL, int PAT, int MASK>
__host__ __device__ constexpr bool kbc_staged() {
    return LGB_KBC_STAGE && SID == LGB_D3Q27 && COLL == LGB_KBC && ST == LGB_F32 &&
           (PAT == LGB_PULL || PAT == LGB_LOCAL) && (MASK == 0 || MASK == 1 || MASK == 3);
}

template <class R> struct StagePops {
    R *col;
    __device__ __forceinline__ R get(int q) const {
        return *reinterpret_cast<volatile R *>(col + q * kStageThreads);
    }
    __device__ __forceinline__ void set(int q, R v) const {
        *reinterpret_cast<volatile R *>(col + q * kStageThreads) = v;
    }
};

// MASK: 0 = no boundaries; 1 = boundaries, every cell except those of the
// anti-bounce-back outlet plane (when there is one); 2 = the outlet plane
// only (one thread per plane cell); 3 and 4 = 1 and 2 with bounce-back links
// (only these variants carry the link code, so the others keep their
// register budget). Splitting the outlet off keeps its extra
// neighbour reconstruction out of the register budget of the bulk launch.
// The step of one cell; the kernels below wrap it with their launch bounds.
template <int SID, int ST, int COLL, int PAT, int MASK, class TT>
__device__ __forceinline__ void step_cell(const StepParams &p, const TT &tab) {
    using S = Stencil<SID>;
    using Sto = Storage<ST>;
    using R = typename Sto::R;
    using T = typename Sto::T;
    constexpr bool MASKED = MASK != 0;
    constexpr bool PLANE = MASK == 2 || MASK == 4;
    constexpr bool BULK = MASK == 1 || MASK == 3;
    constexpr bool LINKS = MASK >= 3;
    constexpr bool SUBSTEPS = PAT != LGB_STREAM_ONLY && PAT != LGB_AA_UNPACK;
    constexpr int LOAD = PatternTraits<PAT>::load;
    // 16-bit formats without boundaries collide in shifted space, with the
    // same arithmetic as the two-cell kernel
    constexpr bool HSPACE = is_shifted<ST>() && !MASKED && shifted_collision<COLL>();
    const T *__restrict__ fin = static_cast<const T *>(p.f_in);
    T *fout = static_cast<T *>(p.f_out);
    uint32_t n, x, y, z;
    if constexpr (PLANE) {
        // plane cell i -> (x, y, z) with the normal coordinate fixed
        const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
        const uint32_t a = p.abb_axis == 0 ? p.Y : p.X;  // first free axis extent
        const uint32_t b = p.abb_axis == 2 ? p.Y : p.Z;  // second (fastest) free axis
        if (i >= a * b) return;
        const uint32_t u0 = i / b, u1 = i - u0 * b;
        if (p.abb_axis == 0) { x = p.abb_plane; y = u0; z = u1; }
        else if (p.abb_axis == 1) { x = u0; y = p.abb_plane; z = u1; }
        else { x = u0; y = u1; z = p.abb_plane; }
        n = (x * p.Y + y) * p.Z + z;
    } else {
        n = blockIdx.x * blockDim.x + threadIdx.x;
        if (n >= p.N) return;
        const uint32_t row = p.divZ.div(n);
        z = n - row * p.Z;
        x = p.divY.div(row);
        y = row - x * p.Y;
    }
    Nbr c;
    c.set(x, y, z, p);
    if constexpr (BULK && SUBSTEPS) {
        // the outlet plane has its own launch
        if (p.abb_k >= 0 && coord_along(c, p.abb_axis) == p.abb_plane) return;
    }

    uint8_t fl = 0;
    uint32_t nsbits = 0, lbits = 0;
    if (MASKED) {
        fl = p.flags[n];
        if ((fl & LGB_FLAG_NO_STREAM) && p.nsb) nsbits = p.nsb[n];
        if (LINKS && LOAD == LOAD_PULL && (fl & LGB_FLAG_LINKS) && p.links) lbits = p.links[n];
    }
    R f[S::Q];
    load_cell<S, Sto, LOAD, MASKED, HSPACE, LINKS>(p, fin, c, n, nsbits, f, lbits);

    if constexpr (kbc_staged<SID, ST, COLL, PAT, MASK>()) {
        // (each thread reads and writes only its own column: no barrier)
        __shared__ R stage[S::Q * kStageThreads];
        const StagePops<R> sp{stage + threadIdx.x};
#pragma unroll
        for (int q = 0; q < S::Q; ++q) sp.set(q, f[q]);
        const int idx = fl & LGB_FLAG_INDEX_MASK;
        if (!BULK || idx == p.coll_idx) {
            R r;
            collide_kbc_of<S>(sp, p.cp, r);
        } else {
            R g[S::Q];
#pragma unroll
            for (int q = 0; q < S::Q; ++q) g[q] = sp.get(q);
            apply_local_substep<S, COLL, false>(p, select_sub(p, idx), c, g, tab);
#pragma unroll
            for (int q = 0; q < S::Q; ++q) sp.set(q, g[q]);
        }
        const size_t N = p.N;
        R r = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) {
            const R v = sp.get(q);
            r += v;
            store_value<Sto, false>(fout + (size_t)q * N + n, v, S::w(q));
        }
        if (p.status && !isfinite(r)) atomicOr(p.status, 1u);
        return;
    }

    if constexpr (HSPACE) {
        if constexpr (PAT != LGB_STREAM_ONLY && PAT != LGB_AA_UNPACK)
            collide_shifted<S, Lane1, COLL>(f, p.cp);
    } else if constexpr (PAT != LGB_STREAM_ONLY && PAT != LGB_AA_UNPACK) {
        if constexpr (BULK) {
            // a cell off the outlet plane runs the substep its index names;
            // the collision (most cells) without copying out a substep record
            const int idx = fl & LGB_FLAG_INDEX_MASK;
            if (idx == p.coll_idx) {
                R r;
                collide<COLL, S>(f, p.cp, r, tab);
            } else {
                apply_local_substep<S, COLL, false>(p, select_sub(p, idx), c, f, tab);
            }
        } else if constexpr (PLANE) {
            // an outlet-plane cell runs the substep its index names and the
            // outlet substep, in sequence order
            const int idx = fl & LGB_FLAG_INDEX_MASK;
            const bool outlet = p.abb_k >= 0 && coord_along(c, p.abb_axis) == p.abb_plane;
            const int outlet_phase = p.abb_k < idx ? 0 : 1;
#pragma unroll 1
            for (int phase = 0; phase < 2; ++phase) {
                if (phase != outlet_phase && idx != p.abb_k)
                    apply_local_substep<S, COLL>(p, select_sub(p, idx), c, f, tab);
                if (phase == outlet_phase && outlet)
                    apply_outlet<S, COLL, LOAD, MASKED, LINKS, Sto>(p, fin, c, f, tab);
            }
        } else {
            R r;
            collide<COLL, S>(f, p.cp, r, tab);
        }
    }

    if (p.status) {
        R r = R(0);
#pragma unroll
        for (int q = 0; q < S::Q; ++q) r += f[q];
        if (!isfinite(r)) atomicOr(p.status, 1u);
    }

    const size_t N = p.N;
    // PUSH with no-streaming bits: this cell keeps some of its own values or
    // writes into a destination that keeps some of its own
    bool guarded = false;
    if constexpr (MASKED && PAT == LGB_PUSH)
        guarded = p.has_nsm &&
                  (!p.push_guard || (fl & (LGB_FLAG_PUSH_GUARD | LGB_FLAG_NO_STREAM)));
#pragma unroll
    for (int q = 0; q < S::Q; ++q) {
        if constexpr (PAT == LGB_PULL || PAT == LGB_LOCAL || PAT == LGB_STREAM_ONLY ||
                      PAT == LGB_AA_UNPACK) {
            store_value<Sto, HSPACE>(fout + (size_t)q * N + n, f[q], S::w(q));
        } else if constexpr (PAT == LGB_AA_EVEN) {
            store_value<Sto, HSPACE>(fout + (size_t)S::opp(q) * N + n, f[q], S::w(q));
        } else {  // PUSH, AA_ODD: to the neighbour in direction e_q, slot q
            const uint32_t dst = c.at(ix<S>(q), iy<S>(q), iz<S>(q), p);
            if (MASKED && PAT == LGB_PUSH && guarded && q != 0) {
                // lettuce keeps the destination's own value where its
                // no-streaming bit is set
                const uint8_t fd = p.flags[dst];
                const bool blocked = (fd & LGB_FLAG_NO_STREAM) && ((p.nsb[dst] >> q) & 1u);
                if (!blocked) store_value<Sto, HSPACE>(fout + (size_t)q * N + dst, f[q], S::w(q));
                if ((nsbits >> q) & 1u) store_value<Sto, HSPACE>(fout + (size_t)q * N + n, f[q], S::w(q));
            } else {
                store_value<Sto, HSPACE>(fout + (size_t)q * N + dst, f[q], S::w(q));
            }
        }
    }
}

// Only a block-size bound: a minimum-blocks bound of 1 lets the compiler
// take more registers (the D3Q19 float32 pull kernel went from 48 to 72
// registers and lost 11 %).
template <int SID, int ST, int COLL>
using StepTables = typename TablesOf<COLL, Stencil<SID>, typename Storage<ST>::R>::type;

template <int SID, int ST, int COLL, int PAT, int MASK>
__global__ void __launch_bounds__(256)
step_kernel(const __grid_constant__ StepParams p, const __grid_constant__ StepTables<SID, ST, COLL> tab) {
    step_cell<SID, ST, COLL, PAT, MASK>(p, tab);
}

// The D3Q27 KBC bulk kernels are held to 64 registers (4 blocks per SM):
// measured on the 512x128x128 obstacle, 22.7k MLUPS against 17.1k with the
// compiler's 80-103 registers, despite a few spilled values. The push
// variant keeps the scatter's neighbours across the collision and does
// better at 80 registers (3 blocks per SM: 22.5k against 21.6k MLUPS).
#ifndef LGB_KBC_MIN_BLOCKS
#define LGB_KBC_MIN_BLOCKS 4
#endif
#ifndef LGB_KBC_PUSH_MIN_BLOCKS
#define LGB_KBC_PUSH_MIN_BLOCKS 3
#endif
// the staged float32 kernels (27.6 KB of shared memory per block)
#ifndef LGB_KBC_STAGE_MIN_BLOCKS
#define LGB_KBC_STAGE_MIN_BLOCKS 4
#endif
template <int SID, int ST, int COLL, int PAT, int MASK>
constexpr int kbc_min_blocks() {
    return kbc_staged<SID, ST, COLL, PAT, MASK>()
               ? LGB_KBC_STAGE_MIN_BLOCKS
               : (PAT == LGB_PUSH ? LGB_KBC_PUSH_MIN_BLOCKS : LGB_KBC_MIN_BLOCKS);
}
template <int SID, int ST, int COLL, int PAT, int MASK>
__global__ void __launch_bounds__(256, (kbc_min_blocks<SID, ST, COLL, PAT, MASK>()))
step_kernel_bounded(const __grid_constant__ StepParams p,
                    const __grid_constant__ StepTables<SID, ST, COLL> tab) {
    step_cell<SID, ST, COLL, PAT, MASK>(p, tab);
}

// the collision's tables for one launch, from the host copy the caller gave
template <int SID, int ST, int COLL>
StepTables<SID, ST, COLL> make_tables(const StepParams &p) {
    StepTables<SID, ST, COLL> t{};
    if constexpr (COLL == LGB_MRT) {
        using R = typename Storage<ST>::R;
        constexpr int Q = Stencil<SID>::Q;
        for (int i = 0; i < Q * Q; ++i) {
            t.M[i] = R(p.mrt_host[i]);
            t.Minv[i] = R(p.mrt_host[Q * Q + i]);
        }
        for (int i = 0; i < Q; ++i) t.inv_s[i] = R(1.0 / p.mrt_host[2 * Q * Q + i]);
        t.eq = p.mrt_eq;
    }
    return t;
}

template <int SID, int ST, int COLL, int PAT, int MASK>
cudaError_t launch_step(const StepParams &p, cudaStream_t stream) {
    // the outlet plane has few cells (128 x 128 for the obstacle): smaller
    // blocks spread them over more SMs
    constexpr bool PLANE = MASK == 2 || MASK == 4;
    const unsigned threads = PLANE ? 64 : 256;
    uint64_t count = p.N;
    if (PLANE) {
        const uint32_t ax = p.abb_axis == 0 ? p.X : (p.abb_axis == 1 ? p.Y : p.Z);
        count = p.N / ax;
    }
    const unsigned blocks = (unsigned)((count + threads - 1) / threads);
    const StepTables<SID, ST, COLL> tab = make_tables<SID, ST, COLL>(p);
    if constexpr (COLL == LGB_KBC && SID == LGB_D3Q27 && !PLANE)
        step_kernel_bounded<SID, ST, COLL, PAT, MASK><<<blocks, threads, 0, stream>>>(p, tab);
    else
        step_kernel<SID, ST, COLL, PAT, MASK><<<blocks, threads, 0, stream>>>(p, tab);
    return cudaGetLastError();
}

// collision kinds that are instantiated for a stencil
template <int SID> constexpr bool has_kbc() { return SID == LGB_D2Q9 || SID == LGB_D3Q27; }

// with boundaries: the bulk launch (MASK 1) and, if there is an outlet and
// the pattern has substeps, the outlet-plane launch (MASK 2)
// A second stream of the current device ordered after `s` (fork), and the
// join of its work back into `s` (lgb_abi.cu). fork_aux returns nullptr
// where no second stream is available; the caller then stays on `s`.
cudaStream_t fork_aux(cudaStream_t s);
cudaError_t join_aux(cudaStream_t s, cudaStream_t aux);

template <int SID, int ST, int COLL, int PAT, int BULK, int PLANE>
cudaError_t launch_masked(const StepParams &p, cudaStream_t s) {
    constexpr bool SUBSTEPS = PAT != LGB_STREAM_ONLY && PAT != LGB_AA_UNPACK;
    constexpr bool OUTLET = SUBSTEPS && PAT != LGB_AA_EVEN && PAT != LGB_AA_ODD;
    if constexpr (OUTLET) {
        if (p.abb_k >= 0) {
            // the outlet plane and the bulk write disjoint populations
            // (every destination slot has one writer) and only read the
            // input field: the short plane launch runs beside the bulk
            cudaStream_t aux = fork_aux(s);
            if (aux) {
                const cudaError_t e2 = launch_step<SID, ST, COLL, PAT, PLANE>(p, aux);
                const cudaError_t e1 = launch_step<SID, ST, COLL, PAT, BULK>(p, s);
                const cudaError_t e3 = join_aux(s, aux);
                return e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
            }
            const cudaError_t e = launch_step<SID, ST, COLL, PAT, BULK>(p, s);
            if (e != cudaSuccess) return e;
            return launch_step<SID, ST, COLL, PAT, PLANE>(p, s);
        }
    }
    return launch_step<SID, ST, COLL, PAT, BULK>(p, s);
}

template <int SID, int ST, int COLL, int PAT, bool MASKED>
cudaError_t launch_step_set(const StepParams &p, cudaStream_t s) {
    if constexpr (!MASKED) {
        return launch_step<SID, ST, COLL, PAT, 0>(p, s);
    } else {
        // bounce-back links act in the pulling patterns only (LGB_LOCAL
        // ignores them)
        if constexpr (PAT == LGB_PULL || PAT == LGB_STREAM_ONLY) {
            if (p.links) return launch_masked<SID, ST, COLL, PAT, 3, 4>(p, s);
        }
        return launch_masked<SID, ST, COLL, PAT, 1, 2>(p, s);
    }
}

// EXT = false: the ABI's base collisions (none, BGK, TRT, KBC); EXT = true:
// forced BGK, regularized, Smagorinsky and MRT. The two sets are instantiated in
// separate translation units so the build compiles them in parallel.
template <int SID, int ST, int PAT, bool MASKED, bool EXT>
cudaError_t dispatch_collision(int coll, const StepParams &p, cudaStream_t s) {
    if constexpr (PAT == LGB_STREAM_ONLY || PAT == LGB_AA_UNPACK) {
        if constexpr (EXT) return cudaErrorInvalidValue;
        else return launch_step_set<SID, ST, LGB_NO_COLLISION, PAT, MASKED>(p, s);
    } else if constexpr (EXT) {
        switch (coll) {
        case LGB_BGK_FORCED: return launch_step_set<SID, ST, LGB_BGK_FORCED, PAT, MASKED>(p, s);
        case LGB_REGULARIZED: return launch_step_set<SID, ST, LGB_REGULARIZED, PAT, MASKED>(p, s);
        case LGB_SMAGORINSKY: return launch_step_set<SID, ST, LGB_SMAGORINSKY, PAT, MASKED>(p, s);
        case LGB_MRT: return launch_step_set<SID, ST, LGB_MRT, PAT, MASKED>(p, s);
        }
        return cudaErrorInvalidValue;
    } else {
        switch (coll) {
        case LGB_NO_COLLISION: return launch_step_set<SID, ST, LGB_NO_COLLISION, PAT, MASKED>(p, s);
        case LGB_BGK: return launch_step_set<SID, ST, LGB_BGK, PAT, MASKED>(p, s);
        case LGB_TRT: return launch_step_set<SID, ST, LGB_TRT, PAT, MASKED>(p, s);
        case LGB_KBC:
            if constexpr (has_kbc<SID>()) return launch_step_set<SID, ST, LGB_KBC, PAT, MASKED>(p, s);
            return cudaErrorNotSupported;
        }
        return cudaErrorInvalidValue;
    }
}

// pattern sets of one instantiation unit: the pulling patterns (the ones
// that carry bounce-back links) and the others
enum PatternSet { PATTERNS_ALL = 0, PATTERNS_PULLING = 1, PATTERNS_OTHER = 2 };
__host__ __device__ constexpr bool pulling_pattern(int pat) {
    return pat == LGB_PULL || pat == LGB_STREAM_ONLY;
}

template <int SID, int ST, bool MASKED, bool EXT, int SET = PATTERNS_ALL>
cudaError_t dispatch_pattern(int coll, int pat, const StepParams &p, cudaStream_t s) {
    constexpr bool PULLING = SET != PATTERNS_OTHER;
    constexpr bool OTHER = SET != PATTERNS_PULLING;
    switch (pat) {
    case LGB_PULL:
        if constexpr (PULLING) return dispatch_collision<SID, ST, LGB_PULL, MASKED, EXT>(coll, p, s);
        break;
    case LGB_STREAM_ONLY:
        if constexpr (PULLING)
            return dispatch_collision<SID, ST, LGB_STREAM_ONLY, MASKED, EXT>(coll, p, s);
        break;
    case LGB_PUSH:
        if constexpr (OTHER) return dispatch_collision<SID, ST, LGB_PUSH, MASKED, EXT>(coll, p, s);
        break;
    case LGB_LOCAL:
        if constexpr (OTHER) return dispatch_collision<SID, ST, LGB_LOCAL, MASKED, EXT>(coll, p, s);
        break;
    case LGB_AA_EVEN:
        if constexpr (OTHER) return dispatch_collision<SID, ST, LGB_AA_EVEN, MASKED, EXT>(coll, p, s);
        break;
    case LGB_AA_ODD:
        if constexpr (OTHER) return dispatch_collision<SID, ST, LGB_AA_ODD, MASKED, EXT>(coll, p, s);
        break;
    case LGB_AA_UNPACK:
        if constexpr (OTHER && !MASKED)
            return dispatch_collision<SID, ST, LGB_AA_UNPACK, false, EXT>(coll, p, s);
        break;
    }
    return cudaErrorInvalidValue;
}

// translation units per (stencil, storage): lgb_step_<stencil>.cu built
// with -DLGB_STORAGE_ID=<storage> and -DLGB_EXT_COLLISIONS=0 (step_*) or 1
// (stepx_*), defining the entries for grids without boundaries (_plain) and
// with them (_masked_pull: PULL and STREAM_ONLY; _masked_rest: the other
// patterns), in one unit or three (-DLGB_MASK_PART)
#define LGB_DECLARE_STEP_PART(name, part)                                                   \
    cudaError_t name##_##part##_s0(int, int, const StepParams &, cudaStream_t);            \
    cudaError_t name##_##part##_s1(int, int, const StepParams &, cudaStream_t);            \
    cudaError_t name##_##part##_s2(int, int, const StepParams &, cudaStream_t);            \
    cudaError_t name##_##part##_s3(int, int, const StepParams &, cudaStream_t);
#define LGB_DECLARE_STEP(name)                                                              \
    LGB_DECLARE_STEP_PART(name, plain)                                                      \
    LGB_DECLARE_STEP_PART(name, masked_pull)                                                \
    LGB_DECLARE_STEP_PART(name, masked_rest)
LGB_DECLARE_STEP(step_d1q3)
LGB_DECLARE_STEP(step_d2q9)
LGB_DECLARE_STEP(step_d3q15)
LGB_DECLARE_STEP(step_d3q19)
LGB_DECLARE_STEP(step_d3q27)
LGB_DECLARE_STEP(stepx_d1q3)
LGB_DECLARE_STEP(stepx_d2q9)
LGB_DECLARE_STEP(stepx_d3q15)
LGB_DECLARE_STEP(stepx_d3q19)
LGB_DECLARE_STEP(stepx_d3q27)
#undef LGB_DECLARE_STEP

}  // namespace lgb
