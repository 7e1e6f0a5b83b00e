// Kernel instantiations for D2Q9 with float population storage.
#define PL_LAT D2Q9
#define PL_STORE float
#define PL_NAME d2q9_f32
#define PL_ALL_KINDS
#define PL_INCOMPRESSIBLE
#define PL_ELASTIC
#include "inst_body.cuh"
