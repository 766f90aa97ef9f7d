// k_ls_energy_f32_c.cu -- line-search energy passes, mixed (FP32) mode, 3, 2, 1 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(float, float, 3)
HX_LS_ENERGY_INST(float, float, 2)
HX_LS_ENERGY_INST(float, float, 1)
}  // namespace hexopt
