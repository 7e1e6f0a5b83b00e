// Kernel instantiations for D2Q9 with __nv_bfloat16 population storage: the collide and fused-step launches of the adjoint inline-boundary kinds.
#define PL_LAT D2Q9
#define PL_STORE __nv_bfloat16
#define PL_NAME d2q9_bf16
#define PL_PART 4
#include "inst_body.cuh"
