// batch_push.cu -- instantiations of the persistent push over many boxes (k_push_tiled_batch,
// Boris pusher), compiled apart from the single-box kernels so they build in parallel.
#include "tiled_kernel.cuh"

namespace osg {

OSG_DEFINE_PUSH_BATCH(OSG_PUSHER_BORIS)

#define OSG_BATCH_OCC(D, O, P)                                                                \
    if (dim == D && order == O) {                                                             \
        int n = 0;                                                                            \
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_push_tiled_batch<D, O, P>,    \
                                                          threads, smem) != cudaSuccess)       \
            return 0;                                                                         \
        return n;                                                                             \
    }

int push_batch_occupancy(int dim, int order, int threads, size_t smem)
{
    OSG_PUSH_TILED_CASES(OSG_PUSHER_BORIS, OSG_BATCH_OCC)
    return 0;
}

} // namespace osg
