// gb_btiled_f.cu -- single-precision dispatch of the tiled B / B^T kernels (the kernels are
// instantiated in gb_btiled_f1.cu .. gb_btiled_f3.cu).
#include "gb_btiled.cuh"
GB_INSTANTIATE_TILED(float)
