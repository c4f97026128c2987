// tiled_condvay.cu -- instantiations of the tiled push kernel with the conditional Vay momentum
// update (dudt_cond_vay, source/spec/os-spec-push.f03:800-1100: Vay above gamma 5, else Boris);
// compiled apart so the kernel sets build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_COND_VAY, push_tiled_launch_cond_vay, push_tiled_attr_cond_vay)

} // namespace osg
