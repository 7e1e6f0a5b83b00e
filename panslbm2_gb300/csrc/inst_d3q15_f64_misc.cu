// Kernel instantiations for D3Q15 with double population storage: the collide and fused-step launches of the other kinds.
#define PL_LAT D3Q15
#define PL_STORE double
#define PL_NAME d3q15_f64
#define PL_ALL_KINDS
#define PL_PART 5
#include "inst_body.cuh"
