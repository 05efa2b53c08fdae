// gb_btiled_d.cu -- double-precision dispatch of the tiled B / B^T kernels (the kernels are
// instantiated in gb_btiled_d1.cu .. gb_btiled_d3.cu).
#include "gb_btiled.cuh"
GB_INSTANTIATE_TILED(double)
