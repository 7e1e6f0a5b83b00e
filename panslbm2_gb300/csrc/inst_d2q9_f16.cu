// Kernel instantiations for D2Q9 with __half population storage.
#define PL_LAT D2Q9
#define PL_STORE __half
#define PL_NAME d2q9_f16

#include "inst_body.cuh"
