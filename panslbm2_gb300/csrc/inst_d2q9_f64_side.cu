// Kernel instantiations for D2Q9 with double population storage: the side-stream boundary kernels.
#define PL_LAT D2Q9
#define PL_STORE double
#define PL_NAME d2q9_f64
#define PL_ALL_KINDS
#define PL_INCOMPRESSIBLE
#define PL_ELASTIC
#define PL_PART 3
#include "inst_body.cuh"
