// Kernel instantiations for D3Q15 with __half population storage: the collide and fused-step launches of the adjoint inline-boundary kinds.
#define PL_LAT D3Q15
#define PL_STORE __half
#define PL_NAME d3q15_f16
#define PL_PART 4
#include "inst_body.cuh"
