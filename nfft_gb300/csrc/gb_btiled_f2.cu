// gb_btiled_f2.cu -- single-precision 2-D instantiations of the tiled B / B^T kernels
// (one translation unit per precision and dimension, so that they compile in parallel).
#include "gb_btiled.cuh"

namespace gb {
GB_TILED_DIM_DECL(, float, 2)
}  // namespace gb
