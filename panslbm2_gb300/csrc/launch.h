// launch.h -- host-side declarations of the per-(lattice, storage) launch switches.
#pragma once
#include <cuda_runtime.h>
#include "common.h"

namespace pl {
enum LaunchOp { OP_COLLIDE = 0, OP_STEP = 1, OP_BOUNDARY = 2, OP_SNAPSHOT = 3 };
enum AuxOp { AUX_STREAM_PROGRAM = 0, AUX_INIT = 1, AUX_DECODE = 2, AUX_ENCODE = 3 };

#define PL_DECL(name)                                                                                   \
    int launch_##name(int kind, int op, bool save, const KArgs &a, cudaStream_t st);                     \
    int launch_adj_##name(int kind, int op, bool save, const KArgs &a, cudaStream_t st);                 \
    int launch_misc_##name(int kind, int op, bool save, const KArgs &a, cudaStream_t st);                \
    void aux_##name(int op, const KArgs &a, int which, const double *const *in, int has_g, int sgn,     \
                    double *buf, int set, double shift, cudaStream_t st);                                \
    void side_step_##name(const KArgs &a, int kind, cudaStream_t side, cudaStream_t side2);             \
    void side_stream_##name(const KArgs &a, cudaStream_t side, cudaStream_t side2);
PL_DECL(d2q9_f64)
PL_DECL(d2q9_f32)
PL_DECL(d2q9_f16)
PL_DECL(d2q9_bf16)
PL_DECL(d3q15_f64)
PL_DECL(d3q15_f32)
PL_DECL(d3q15_f16)
PL_DECL(d3q15_bf16)
#undef PL_DECL

// records the message pl_last_error returns (for entry points defined outside api.cu)
int record_error(int code, const char *msg);
}  // namespace pl

typedef struct pl_lattice_s *pl_lattice;
namespace pl {
// device pointers of a lattice's frozen forward solution (rho, ux, uy, uz, T) and last saved
// adjoint macros (ip, iux, iuy, iuz, iT, iqx, iqy, iqz); unused planes are NULL
int lattice_sample_fields(pl_lattice h, const double **p, long long *n);
cudaStream_t lattice_stream(pl_lattice h);
}  // namespace pl
