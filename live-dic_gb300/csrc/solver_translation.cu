// IC-GN solver instantiations for the translation model (see solver_impl.cuh).
#include "gbdic_kernels.h"
#include "solver_impl.cuh"

namespace gbdic {
GBDIC_SOLVER_MODEL(kModelTranslation)
}  // namespace gbdic
