// Instantiations of the step kernels for D3Q15; compiled once per
// population storage (-DLGB_STORAGE_ID=0..3) so the build runs them in
// parallel. The two-cell kernel exists for the 16-bit storages (2, 3).
#include "lgb_step.cuh"
#include "lgb_step_vec.cuh"

#ifndef LGB_STORAGE_ID
#error "compile with -DLGB_STORAGE_ID=<storage>"
#endif
#ifndef LGB_EXT_COLLISIONS
#define LGB_EXT_COLLISIONS 0
#endif
#define LGB_CAT2(a, b) a##b
#define LGB_CAT(a, b) LGB_CAT2(a, b)

namespace lgb {
#if LGB_EXT_COLLISIONS
cudaError_t LGB_CAT(stepx_d3q15_s, LGB_STORAGE_ID)(int coll, int pat, bool masked,
                                                   const StepParams &p, cudaStream_t s) {
    return masked ? dispatch_pattern<LGB_D3Q15, LGB_STORAGE_ID, true, true>(coll, pat, p, s)
                  : dispatch_pattern<LGB_D3Q15, LGB_STORAGE_ID, false, true>(coll, pat, p, s);
}
#else
cudaError_t LGB_CAT(step_d3q15_s, LGB_STORAGE_ID)(int coll, int pat, bool masked,
                                                  const StepParams &p, cudaStream_t s) {
    return masked ? dispatch_pattern<LGB_D3Q15, LGB_STORAGE_ID, true, false>(coll, pat, p, s)
                  : dispatch_pattern<LGB_D3Q15, LGB_STORAGE_ID, false, false>(coll, pat, p, s);
}
#if LGB_STORAGE_ID >= 2
cudaError_t LGB_CAT(step_vec2_d3q15_s, LGB_STORAGE_ID)(int coll, int pat, const StepParams &p,
                                                       cudaStream_t s) {
    return dispatch_vec2<LGB_D3Q15, LGB_STORAGE_ID>(coll, pat, p, s);
}
#endif
#endif  // LGB_EXT_COLLISIONS
}  // namespace lgb
