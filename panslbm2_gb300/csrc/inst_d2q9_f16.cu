// Kernel instantiations for D2Q9 with __half population storage: the launch switch and the collide and fused-step launches of the forward inline-boundary kinds.
#define PL_LAT D2Q9
#define PL_STORE __half
#define PL_NAME d2q9_f16
#define PL_PART 1
#include "inst_body.cuh"
