// gb_btiled_d.cu -- double-precision instantiations of the tiled B / B^T kernels.
#include "gb_btiled.cuh"
GB_INSTANTIATE_TILED(double)
