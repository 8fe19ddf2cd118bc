// Batched element operator instantiations for lx1 = 4.
#include "nb_batch_ax.cuh"

namespace nb {
NB_BATCH_AX_INSTANTIATE(4)
}  // namespace nb
