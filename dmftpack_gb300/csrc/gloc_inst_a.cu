// gloc_inst_a.cu -- explicit instantiations of k_gloc (split for a parallel build).
#include "gloc.cuh"

namespace dg {
DG_GLOC_INST(1, 1)
DG_GLOC_INST(2, 2)
DG_GLOC_INST(3, 4)
DG_GLOC_INST(4, 4)
}  // namespace dg
