// density_inst.cu -- explicit instantiations of k_dens_sum (density.cuh), the lane-group widths of k_schur.
#include "density.cuh"

namespace dg {
DG_DENS_INST(1, 1)
DG_DENS_INST(2, 2)
DG_DENS_INST(3, 4)
DG_DENS_INST(4, 4)
DG_DENS_INST(6, 8)
DG_DENS_INST(8, 8)
DG_DENS_INST(10, 16)
DG_DENS_INST(12, 16)
DG_DENS_INST(16, 16)
DG_DENS_INST(20, 32)
}  // namespace dg
