// schur_inst_d.cu -- explicit instantiations of k_schur (split for a parallel build).
#include "schur.cuh"

namespace dg {
DG_SCHUR_INST(16, 16)
}  // namespace dg
