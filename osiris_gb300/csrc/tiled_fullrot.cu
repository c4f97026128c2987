// tiled_fullrot.cu -- instantiations of the tiled push kernel with the full-rotation momentum update (dudt_fullrot,
// source/spec/os-spec-push.f03:83-231);
// compiled apart so the kernel sets build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_FULLROT, push_tiled_launch_fullrot, push_tiled_attr_fullrot)

} // namespace osg
