// tiled_exact.cu -- instantiations of the tiled push kernel with the exact momentum update
// (push_type = "exact", dudt_exact, source/spec/os-spec-extpush.f03:40-348); compiled apart
// from tiled.cu so the two halves of the kernel set build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_TILED(OSG_PUSHER_EXACT, push_tiled_launch_exact, push_tiled_attr_exact)

} // namespace osg
