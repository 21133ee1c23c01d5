// schur_tpi.cu -- instantiations of the thread-per-frequency BLOCK kernel k_schur_tpi (schur.cuh), D = 1 .. 3.
#include "schur.cuh"

namespace dg {
SchurKernel schur_tpi_kernel(int D, bool mixed) {
    switch (D) {
        case 1: return mixed ? k_schur_tpi<OpsF, 1> : k_schur_tpi<OpsD, 1>;
        case 2: return mixed ? k_schur_tpi<OpsF, 2> : k_schur_tpi<OpsD, 2>;
        case 3: return mixed ? k_schur_tpi<OpsF, 3> : k_schur_tpi<OpsD, 3>;
    }
    return nullptr;
}
}  // namespace dg
