// k_stubs3d.cu -- entry points of physics whose fused kernels are not in
// this build; they fail loudly with GPI_E_UNSUPPORTED.
#include "gpi_internal.cuh"

namespace gpi {

int step_acoustic3d(Plan *p, int, int, int, int) {
  return fail(p, GPI_E_UNSUPPORTED, "3-D acoustic kernels are not part of this build");
}
int step_elastic3d(Plan *p, int, int, int, int) {
  return fail(p, GPI_E_UNSUPPORTED, "3-D elastic kernels are not part of this build");
}

}  // namespace gpi
