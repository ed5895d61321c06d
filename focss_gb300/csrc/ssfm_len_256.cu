// ssfm_len_256.cu -- instantiation of the split-step passes for length-256 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(256, 8)
FG_INSTANTIATE_ROW(256, 8)
