// k_ls_energy_f64_c.cu -- line-search energy passes, FP64 mode, 3, 2, 1 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(double, double, 3)
HX_LS_ENERGY_INST(double, double, 2)
HX_LS_ENERGY_INST(double, double, 1)
}  // namespace hexopt
