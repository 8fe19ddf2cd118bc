// Batched element operator instantiations for lx1 = 12.
#include "nb_batch_ax.cuh"

namespace nb {
NB_BATCH_AX_INSTANTIATE(12)
}  // namespace nb
