// tcgen05 BF16x3 transform contractions (placeholder until the tensor-core path lands).
#include "../../include/aieplace.h"
#include "ap_kernels.h"

namespace ap {

int field_solve_bf16x3(FieldSolver &f, const __nv_bfloat16 *d_hi, const __nv_bfloat16 *d_lo, float *ex,
                       float *ey, cudaStream_t st) {
    (void)f; (void)d_hi; (void)d_lo; (void)ex; (void)ey; (void)st;
    return AP_ERR_UNSUPPORTED;
}

}  // namespace ap
