// Batched element operator instantiations for lx1 = 10.
#include "nb_batch_ax.cuh"

namespace nb {
NB_BATCH_AX_INSTANTIATE(10)
}  // namespace nb
