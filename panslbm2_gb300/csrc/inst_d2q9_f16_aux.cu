// Kernel instantiations for D2Q9 with __half population storage: the auxiliary launches (standalone stream, init, host transfer).
#define PL_LAT D2Q9
#define PL_STORE __half
#define PL_NAME d2q9_f16
#define PL_PART 2
#include "inst_body.cuh"
