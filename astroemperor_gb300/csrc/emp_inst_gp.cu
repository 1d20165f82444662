// Instantiations of the celerite GP kernel by state dimension (separate
// translation unit so that it compiles in parallel with the others).
#include "emp_gp.cuh"

namespace emp {

using KFn = void (*)(KArgs);

template <int M>
static KFn pick_gp(int prep, int ff) {
    if (ff) return k_gp_fused<M>;
    return prep ? k_gp_prep<M> : k_gp<M>;
}

// FP64: the recursion kernel of M state dimensions, or (prep != 0) its
// parallel preparation kernel; ff != 0 (mixed precision): the preparation and
// the float-float recursion in one kernel
KFn get_kernel_gp(int M, int prep, int ff) {
    switch (M) {
        case 2: return pick_gp<2>(prep, ff);
        case 4: return pick_gp<4>(prep, ff);
        case 8: return pick_gp<8>(prep, ff);
        case 16: return pick_gp<16>(prep, ff);
        default: return nullptr;
    }
}

}  // namespace emp
