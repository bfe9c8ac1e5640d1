// Split-precision form for complex64 contexts (placeholder until the kernels land).
#include <math.h>

#include "ctx.h"

namespace pgb {

int split_order(double hnorm, double h, long long P) {
    (void)P;
    return select_cycles(true, hnorm, h);
}

Parament_ErrorCode run_split(Ctx *, const void *, unsigned, unsigned, double, int, long long, void *, cudaStream_t) {
    return PARAMENT_STATUS_INVALID_VALUE;
}

}  // namespace pgb
