// ssfm_len_32.cu -- instantiation of the split-step passes for length-32 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(32, 5)
FG_INSTANTIATE_ROW(32, 5)
