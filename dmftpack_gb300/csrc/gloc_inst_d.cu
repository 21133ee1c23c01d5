// gloc_inst_d.cu -- explicit instantiations of k_gloc (split for a parallel build).
#include "gloc.cuh"

namespace dg {
DG_GLOC_INST(16, 16)
}  // namespace dg
