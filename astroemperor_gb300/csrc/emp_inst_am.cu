// The astrometric term of the joint RV + astrometry likelihood (own
// translation unit).
#include "emp_am.cuh"

namespace emp {

using KFn = void (*)(KArgs);

// the astrometric kernel of a precision (EMP_PREC_FP64 or EMP_PREC_MIXED)
KFn get_kernel_am(int prec) { return prec == EMP_PREC_MIXED ? k_am<EMP_PREC_MIXED> : k_am<EMP_PREC_FP64>; }

}  // namespace emp
