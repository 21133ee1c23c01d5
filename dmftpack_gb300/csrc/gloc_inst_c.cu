// gloc_inst_c.cu -- explicit instantiations of k_gloc (split for a parallel build).
#include "gloc.cuh"

namespace dg {
DG_GLOC_INST(12, 16)
}  // namespace dg
