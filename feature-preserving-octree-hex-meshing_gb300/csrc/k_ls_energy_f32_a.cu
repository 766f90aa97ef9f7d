// k_ls_energy_f32_a.cu -- line-search energy passes, mixed (FP32) mode, 8, 7 candidate steps per pass.
#include "k_slim.cuh"

namespace hexopt {
HX_LS_ENERGY_INST(float, float, 8)
HX_LS_ENERGY_INST(float, float, 7)
}  // namespace hexopt
