// FP32-split 3D step (placeholder until the split kernels land).
#include "sim.cuh"

namespace mlau {
struct SplitFields {};
int split3d_alloc(Sim *) { set_error("FP32-split mode is not built yet"); return MLAU_ERR_ARG; }
int split3d_step(Sim *, double) { set_error("FP32-split mode is not built yet"); return MLAU_ERR_ARG; }
void split3d_free(Sim *) {}
}  // namespace mlau
