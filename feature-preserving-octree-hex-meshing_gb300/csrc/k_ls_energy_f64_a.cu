// k_ls_energy_f64_a.cu -- line-search energy passes, FP64 mode, 8, 7 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(double, double, 8)
HX_LS_ENERGY_INST(double, double, 7)
}  // namespace hexopt
