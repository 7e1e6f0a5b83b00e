//  mma.h -- not part of the GPU path: forwards to the reference's own header. Build with
//  -DPANSLBM2_REF=<the reference's source tree> to use it.
#pragma once
#ifndef PANSLBM2_REF
#error "mma.h is the reference's own host code: define PANSLBM2_REF as the path of the reference's source tree"
#endif
#define PANSLBM2_GPU_STR2(x) #x
#define PANSLBM2_GPU_STR(x) PANSLBM2_GPU_STR2(x)
#include PANSLBM2_GPU_STR(PANSLBM2_REF/src/utility/mma.h)
