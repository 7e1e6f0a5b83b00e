// Kernel instantiations for D2Q9 with float population storage: the launch switch and the collide and fused-step launches of the forward inline-boundary kinds.
#define PL_LAT D2Q9
#define PL_STORE float
#define PL_NAME d2q9_f32
#define PL_ALL_KINDS
#define PL_INCOMPRESSIBLE
#define PL_ELASTIC
#define PL_PART 1
#include "inst_body.cuh"
