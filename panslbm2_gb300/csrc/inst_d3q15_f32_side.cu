// Kernel instantiations for D3Q15 with float population storage: the side-stream boundary kernels.
#define PL_LAT D3Q15
#define PL_STORE float
#define PL_NAME d3q15_f32
#define PL_ALL_KINDS
#define PL_PART 3
#include "inst_body.cuh"
