// ssfm_len_16.cu -- instantiation of the split-step passes for length-16 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(16, 4)
FG_INSTANTIATE_ROW(16, 4)
