// tiled_euler.cu -- instantiations of the tiled push kernel with the Euler-rotation momentum update (dudt_euler,
// source/spec/os-spec-push.f03:235-352);
// compiled apart so the kernel sets build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_EULER, push_tiled_launch_euler, push_tiled_attr_euler)

} // namespace osg
