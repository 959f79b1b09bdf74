// Mixed form: FP32 Jacobians, Schur blocks and PCG vectors; FP64 cost, PCG
// inner products and 3x3 / 6x6 block inversions.
#include "runner.cuh"

namespace ba {
template void run_lm<float>(Context&, const Opts&);
template void debug_lm_step<float>(Context&, const Opts&, double, double*, double*, double*,
                                   int32_t*, double*);
}
