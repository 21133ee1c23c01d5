// adjoint_inst.cu -- explicit instantiations of k_gloc_ad (adjoint.cuh), one translation unit for all widths.
#include "adjoint.cuh"

namespace dg {
DG_AD_INST(1, 1)
DG_AD_INST(2, 2)
DG_AD_INST(3, 4)
DG_AD_INST(4, 4)
DG_AD_INST(6, 8)
DG_AD_INST(8, 8)
DG_AD_INST(10, 16)
DG_AD_INST(12, 16)
DG_AD_INST(16, 16)
DG_AD_INST(20, 32)
}  // namespace dg
