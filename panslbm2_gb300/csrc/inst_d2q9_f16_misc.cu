// Kernel instantiations for D2Q9 with __half population storage: the collide and fused-step launches of the other kinds.
#define PL_LAT D2Q9
#define PL_STORE __half
#define PL_NAME d2q9_f16
#define PL_PART 5
#include "inst_body.cuh"
