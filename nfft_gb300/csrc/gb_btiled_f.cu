// gb_btiled_f.cu -- single-precision instantiations of the tiled B / B^T kernels.
#include "gb_btiled.cuh"
GB_INSTANTIATE_TILED(float)
