// Instantiations of the adjoint kernel (own translation unit).
#include "emp_grad.cuh"

namespace emp {

using GFn = void (*)(GArgs);

template <int Q>
static GFn pick_grad(int lidx) {
    switch (lidx) {
        case 0: return k_grad<Q, 32, 128>;
        default: return nullptr;
    }
}

GFn get_kernel_grad(int q, int lidx) {
    switch (q) {
        case 0: return pick_grad<0>(lidx);
        case 1: return pick_grad<1>(lidx);
        case 2: return pick_grad<2>(lidx);
        case 3: return pick_grad<3>(lidx);
        default: return nullptr;
    }
}

}  // namespace emp
