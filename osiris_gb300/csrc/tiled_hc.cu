// tiled_hc.cu -- instantiations of the tiled push kernel with the Higuera-Cary momentum update (dudt_cary,
// source/spec/os-spec-push.f03:1104-1253);
// compiled apart so the kernel sets build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_HC, push_tiled_launch_hc, push_tiled_attr_hc)

} // namespace osg
