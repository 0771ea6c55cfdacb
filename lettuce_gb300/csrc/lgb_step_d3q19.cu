// Instantiations of the step kernels for D3Q19; compiled once per
// population storage (-DLGB_STORAGE_ID=0..3), per collision set
// (-DLGB_EXT_COLLISIONS=0|1) and, for the large stencils, per part
// (-DLGB_MASK_PART=0: grids without boundaries; 1: with boundaries, the
// pulling patterns; 3: with boundaries, the other patterns; 2, the default:
// all), so the build runs them in parallel. The two-cell kernel exists for
// the 16-bit storages (2, 3) on grids without boundaries.
#include "lgb_step.cuh"
#include "lgb_step_vec.cuh"

#ifndef LGB_STORAGE_ID
#error "compile with -DLGB_STORAGE_ID=<storage>"
#endif
#ifndef LGB_EXT_COLLISIONS
#define LGB_EXT_COLLISIONS 0
#endif
#ifndef LGB_MASK_PART
#define LGB_MASK_PART 2
#endif
#define LGB_CAT2(a, b) a##b
#define LGB_CAT(a, b) LGB_CAT2(a, b)
#define LGB_PART_PLAIN (LGB_MASK_PART == 0 || LGB_MASK_PART == 2)
#define LGB_PART_PULL (LGB_MASK_PART == 1 || LGB_MASK_PART == 2)
#define LGB_PART_REST (LGB_MASK_PART == 3 || LGB_MASK_PART == 2)
#if LGB_EXT_COLLISIONS
#define LGB_ENTRY(part) LGB_CAT(LGB_CAT(stepx_d3q19_, part), LGB_CAT(_s, LGB_STORAGE_ID))
#else
#define LGB_ENTRY(part) LGB_CAT(LGB_CAT(step_d3q19_, part), LGB_CAT(_s, LGB_STORAGE_ID))
#endif

namespace lgb {
#if LGB_PART_PLAIN
cudaError_t LGB_ENTRY(plain)(int coll, int pat, const StepParams &p, cudaStream_t s) {
    return dispatch_pattern<LGB_D3Q19, LGB_STORAGE_ID, false, LGB_EXT_COLLISIONS>(coll, pat, p, s);
}
#if !LGB_EXT_COLLISIONS && LGB_STORAGE_ID >= 2
cudaError_t LGB_CAT(step_vec2_d3q19_s, LGB_STORAGE_ID)(int coll, int pat, const StepParams &p,
                                       cudaStream_t s) {
    return dispatch_vec2<LGB_D3Q19, LGB_STORAGE_ID>(coll, pat, p, s);
}
#endif
#endif
#if LGB_PART_PULL
cudaError_t LGB_ENTRY(masked_pull)(int coll, int pat, const StepParams &p, cudaStream_t s) {
    return dispatch_pattern<LGB_D3Q19, LGB_STORAGE_ID, true, LGB_EXT_COLLISIONS, PATTERNS_PULLING>(
        coll, pat, p, s);
}
#endif
#if LGB_PART_REST
cudaError_t LGB_ENTRY(masked_rest)(int coll, int pat, const StepParams &p, cudaStream_t s) {
    return dispatch_pattern<LGB_D3Q19, LGB_STORAGE_ID, true, LGB_EXT_COLLISIONS, PATTERNS_OTHER>(
        coll, pat, p, s);
}
#endif
}  // namespace lgb
