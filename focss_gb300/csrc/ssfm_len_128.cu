// ssfm_len_128.cu -- instantiation of the split-step passes for length-128 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(128, 7)
FG_INSTANTIATE_ROW(128, 7)
