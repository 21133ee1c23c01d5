// gloc_inst_e.cu -- explicit instantiations of k_gloc (split for a parallel build).
#include "gloc.cuh"

namespace dg {
DG_GLOC_INST(28, 32)
}  // namespace dg
