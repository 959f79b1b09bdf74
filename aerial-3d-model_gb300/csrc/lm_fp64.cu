// Plain form: FP64 throughout.
#include "runner.cuh"

namespace ba {
template void run_lm<double>(Context&, const Opts&);
template void debug_lm_step<double>(Context&, const Opts&, double, double*, double*, double*,
                                    int32_t*, double*);
}
