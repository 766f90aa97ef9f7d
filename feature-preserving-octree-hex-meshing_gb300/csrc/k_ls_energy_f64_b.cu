// k_ls_energy_f64_b.cu -- line-search energy passes, FP64 mode, 6, 5, 4 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(double, double, 6)
HX_LS_ENERGY_INST(double, double, 5)
HX_LS_ENERGY_INST(double, double, 4)
}  // namespace hexopt
