// Instantiations of the celerite GP kernel by state dimension (separate
// translation unit so that it compiles in parallel with the others).
#include "emp_gp.cuh"

namespace emp {

using KFn = void (*)(KArgs);

// the recursion kernel of M state dimensions, or (prep != 0) its parallel
// preparation kernel
KFn get_kernel_gp(int M, int prep) {
    switch (M) {
        case 2: return prep ? k_gp_prep<2> : k_gp<2>;
        case 4: return prep ? k_gp_prep<4> : k_gp<4>;
        case 8: return prep ? k_gp_prep<8> : k_gp<8>;
        case 16: return prep ? k_gp_prep<16> : k_gp<16>;
        default: return nullptr;
    }
}

}  // namespace emp
