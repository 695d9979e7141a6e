// Device code of the reference's 1d2r kernel (src/1d/gpu_2r.cu) as a loadable
// cubin (see ref_cubin_1d1r.cu). Test and baseline infrastructure.
#include "1d_utils.h"
__constant__ double param_matrix_d[2 * 8 * TENSOR_CORE_M];
#include "gpu_2r.cu"
