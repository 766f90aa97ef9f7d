// k_ls_energy_f32_b.cu -- line-search energy passes, mixed (FP32) mode, 6, 5, 4 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(float, float, 6)
HX_LS_ENERGY_INST(float, float, 5)
HX_LS_ENERGY_INST(float, float, 4)
}  // namespace hexopt
