// The astrometric term of the joint RV + astrometry likelihood (own
// translation unit).
#include "emp_am.cuh"

namespace emp {

using KFn = void (*)(KArgs);

KFn get_kernel_am() { return k_am; }

}  // namespace emp
