// gloc_inst_b.cu -- explicit instantiations of k_gloc (split for a parallel build).
#include "gloc.cuh"

namespace dg {
DG_GLOC_INST(6, 8)
DG_GLOC_INST(8, 8)
}  // namespace dg
