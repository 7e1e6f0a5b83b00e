// Kernel instantiations for D2Q9 with double population storage: the auxiliary launches (standalone stream, init, host transfer).
#define PL_LAT D2Q9
#define PL_STORE double
#define PL_NAME d2q9_f64
#define PL_ALL_KINDS
#define PL_INCOMPRESSIBLE
#define PL_ELASTIC
#define PL_PART 2
#include "inst_body.cuh"
