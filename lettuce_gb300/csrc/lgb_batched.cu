// Batched persistent step (lgb_batched_step) and its host-side tile planner
// (lgb_batch_plan); see lgb_batched.cuh.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "lettuce_gb300.h"
#include "lgb_batched.cuh"

namespace lgb {
// the error text of the last failing call lives in lgb_abi.cu
int set_error(const char *msg);
}

namespace {

int bfail(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lgb::set_error(buf);
}

int stencil_d(int s) {
    switch (s) {
    case LGB_D1Q3: return 1;
    case LGB_D2Q9: return 2;
    case LGB_D3Q15: case LGB_D3Q19: case LGB_D3Q27: return 3;
    }
    return 0;
}

}  // namespace

extern "C" {

int lgb_batch_plan(int32_t stencil, int32_t n_domains, const lgb_batch_domain *domains,
                   int32_t tile_cells, lgb_batch_tile *tiles, int32_t max_tiles,
                   int32_t *n_tiles) {
    const int d = stencil_d(stencil);
    if (!d) return bfail("lgb_batch_plan: unknown stencil id %d", stencil);
    if (n_domains < 0 || (n_domains > 0 && !domains) || !n_tiles)
        return bfail("lgb_batch_plan: invalid domain table");
    if (tile_cells < 1) return bfail("lgb_batch_plan: tile_cells must be positive");
    int64_t count = 0;
    for (int b = 0; b < n_domains; ++b) {
        uint64_t rows = 1, z = 0;
        for (int i = 0; i < d; ++i) {
            if (domains[b].res[i] <= 0)
                return bfail("lgb_batch_plan: domain %d has resolution[%d] = %d", b, i,
                             domains[b].res[i]);
            if (i == d - 1) z = (uint64_t)domains[b].res[i];
            else rows *= (uint64_t)domains[b].res[i];
        }
        if (rows * z >= (1ull << 32)) return bfail("lgb_batch_plan: domain %d too large", b);
        const uint64_t per = z >= (uint64_t)tile_cells ? 1 : (uint64_t)tile_cells / z;
        for (uint64_t r = 0; r < rows; r += per) {
            if (tiles) {
                if (count >= max_tiles)
                    return bfail("lgb_batch_plan: more than max_tiles = %d tiles", max_tiles);
                lgb_batch_tile &t = tiles[count];
                t.domain = b;
                t.row_begin = (int32_t)r;
                t.row_end = (int32_t)(r + per < rows ? r + per : rows);
                t.reserved = 0;
            }
            ++count;
        }
    }
    if (count > 0x7fffffff) return bfail("lgb_batch_plan: too many tiles");
    *n_tiles = (int32_t)count;
    return 0;
}

int lgb_batched_step(const lgb_batch_desc *d, void *stream) {
    if (!d) return bfail("lgb_batched_step: descriptor is NULL");
    if (d->abi_version != LGB_ABI_VERSION)
        return bfail("lgb_batched_step: descriptor ABI version %d, library %d", d->abi_version,
                     LGB_ABI_VERSION);
    if (!stencil_d(d->stencil)) return bfail("lgb_batched_step: unknown stencil id %d", d->stencil);
    if (d->storage < LGB_F64 || d->storage > LGB_BF16_SHIFTED)
        return bfail("lgb_batched_step: unknown storage id %d", d->storage);
    if (!(d->collision == LGB_NO_COLLISION || d->collision == LGB_BGK || d->collision == LGB_TRT))
        return bfail("lgb_batched_step: batched domains take BGK, TRT or no collision");
    if (d->n_domains < 1 || d->n_tiles < 1 || !d->domains || !d->tiles)
        return bfail("lgb_batched_step: empty domain or tile table");
    if (!d->f_in || !d->f_out || d->f_in == d->f_out)
        return bfail("lgb_batched_step: needs distinct input and output pools");
    if (d->pool_elements <= 0) return bfail("lgb_batched_step: pool_elements must be positive");
    if (d->threads < 32 || d->threads > 512 || d->threads % 32)
        return bfail("lgb_batched_step: threads = %d (a multiple of 32 up to 512)", d->threads);
    if (d->blocks < 1) return bfail("lgb_batched_step: blocks must be positive");
    lgb::BatchParams p;
    p.f_in = d->f_in;
    p.f_out = d->f_out;
    p.domains = d->domains;
    p.tiles = d->tiles;
    p.n_domains = d->n_domains;
    p.n_tiles = d->n_tiles;
    p.pool_elements = d->pool_elements;
    p.status = d->status;
    if (d->rates && (reinterpret_cast<uintptr_t>(d->rates) & 15u))
        return bfail("lgb_batched_step: rates must be 16-byte aligned");
    p.rates = d->storage == LGB_F64 ? nullptr : reinterpret_cast<const float4 *>(d->rates);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaErrorInvalidValue;
    switch (d->stencil) {
    case LGB_D1Q3: e = lgb::dispatch_batched<LGB_D1Q3>(d->storage, d->collision, p, d->blocks, d->threads, s); break;
    case LGB_D2Q9: e = lgb::dispatch_batched<LGB_D2Q9>(d->storage, d->collision, p, d->blocks, d->threads, s); break;
    case LGB_D3Q15: e = lgb::dispatch_batched<LGB_D3Q15>(d->storage, d->collision, p, d->blocks, d->threads, s); break;
    case LGB_D3Q19: e = lgb::dispatch_batched<LGB_D3Q19>(d->storage, d->collision, p, d->blocks, d->threads, s); break;
    case LGB_D3Q27: e = lgb::dispatch_batched<LGB_D3Q27>(d->storage, d->collision, p, d->blocks, d->threads, s); break;
    }
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "lgb_batched_step: launch failed: %s", cudaGetErrorString(e));
        return lgb::set_error(buf);
    }
    return 0;
}

}  // extern "C"
