// Device code of the reference's 1d1r kernel (src/1d/gpu_1r.cu) as a loadable
// cubin: the reference defines param_matrix_d in main.cu and declares it
// extern in gpu_1r.cu; here the definition precedes the include so the file
// compiles without relocatable device code. Test and baseline infrastructure.
#include "1d_utils.h"
__constant__ double param_matrix_d[2 * 8 * TENSOR_CORE_M];
#include "gpu_1r.cu"
