// Batched element operator instantiations for lx1 = 6.
#include "nb_batch_ax.cuh"

namespace nb {
NB_BATCH_AX_INSTANTIATE(6)
}  // namespace nb
