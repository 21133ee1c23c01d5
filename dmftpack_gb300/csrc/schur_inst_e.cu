// schur_inst_e.cu -- explicit instantiations of k_schur (split for a parallel build).
#include "schur.cuh"

namespace dg {
DG_SCHUR_INST(20, 32)
}  // namespace dg
