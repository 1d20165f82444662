// Instantiations of the celerite GP kernel by state dimension (separate
// translation unit so that it compiles in parallel with the others).
#include "emp_gp.cuh"

namespace emp {

using KFn = void (*)(KArgs);

KFn get_kernel_gp(int M) {
    switch (M) {
        case 2: return k_gp<2>;
        case 4: return k_gp<4>;
        case 8: return k_gp<8>;
        case 16: return k_gp<16>;
        default: return nullptr;
    }
}

}  // namespace emp
