// tiled_vay.cu -- instantiations of the tiled push kernel with the Vay momentum update (dudt_vay, source/spec/os-spec-push.f03:636-796);
// compiled apart so the kernel sets build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_VAY, push_tiled_launch_vay, push_tiled_attr_vay)

} // namespace osg
