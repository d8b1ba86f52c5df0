// k_adjoint2d.cu -- placeholder of the fused adjoint step (built next).
#include "gpi_internal.cuh"

namespace gpi {

int step_adjoint_acoustic2d(Plan *p, int) {
  return fail(p, GPI_E_UNSUPPORTED, "the adjoint step is not part of this build");
}

}  // namespace gpi
