// Kernel instantiations for D3Q15 with __half population storage: the collide and fused-step launches of the other kinds.
#define PL_LAT D3Q15
#define PL_STORE __half
#define PL_NAME d3q15_f16
#define PL_PART 5
#include "inst_body.cuh"
