// schur_inst_c.cu -- explicit instantiations of k_schur (split for a parallel build).
#include "schur.cuh"

namespace dg {
DG_SCHUR_INST(10, 10)
DG_SCHUR_INST(12, 16)
}  // namespace dg
