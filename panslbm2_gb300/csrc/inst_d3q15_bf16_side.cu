// Kernel instantiations for D3Q15 with __nv_bfloat16 population storage: the side-stream boundary kernels.
#define PL_LAT D3Q15
#define PL_STORE __nv_bfloat16
#define PL_NAME d3q15_bf16
#define PL_PART 3
#include "inst_body.cuh"
