// schur_inst_a.cu -- explicit instantiations of k_schur (split for a parallel build).
#include "schur.cuh"

namespace dg {
DG_SCHUR_INST(1, 1)
DG_SCHUR_INST(2, 2)
DG_SCHUR_INST(3, 4)
DG_SCHUR_INST(4, 4)
}  // namespace dg
