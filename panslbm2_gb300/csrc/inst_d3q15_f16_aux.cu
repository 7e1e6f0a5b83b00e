// Kernel instantiations for D3Q15 with __half population storage: the auxiliary launches (standalone stream, init, host transfer).
#define PL_LAT D3Q15
#define PL_STORE __half
#define PL_NAME d3q15_f16
#define PL_PART 2
#include "inst_body.cuh"
