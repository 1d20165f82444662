// Instantiations of the log-posterior kernel for precision EMP_PREC_MIXED
// (separate translation unit so the two precisions compile in parallel).
#include "emp_kernels.cuh"

namespace emp {

using KFn = void (*)(KArgs);

template <int Q>
static KFn pick_mixed(int lidx) {
    switch (lidx) {
        case 0: return k_logpost<EMP_PREC_MIXED, Q, 8, 128>;
        case 1: return k_logpost<EMP_PREC_MIXED, Q, 16, 128>;
        case 2: return k_logpost<EMP_PREC_MIXED, Q, 32, 128>;
        case 3: return k_logpost<EMP_PREC_MIXED, Q, 64, 128>;
        case 4: return k_logpost<EMP_PREC_MIXED, Q, 128, 128>;
        case 5: return k_logpost<EMP_PREC_MIXED, Q, 256, 256>;
        default: return nullptr;
    }
}

KFn get_kernel_mixed(int q, int lidx) {
    switch (q) {
        case 0: return pick_mixed<0>(lidx);
        case 1: return pick_mixed<1>(lidx);
        case 2: return pick_mixed<2>(lidx);
        case 3: return pick_mixed<3>(lidx);
        default: return nullptr;
    }
}

}  // namespace emp
