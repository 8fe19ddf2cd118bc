// Batched element operator instantiations for lx1 = 8.
#include "nb_batch_ax.cuh"

namespace nb {
NB_BATCH_AX_INSTANTIATE(8)
}  // namespace nb
