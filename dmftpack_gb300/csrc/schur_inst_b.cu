// schur_inst_b.cu -- explicit instantiations of k_schur (split for a parallel build).
#include "schur.cuh"

namespace dg {
DG_SCHUR_INST(6, 8)
DG_SCHUR_INST(8, 8)
}  // namespace dg
