// ssfm_len_1024.cu -- instantiation of the split-step passes for length-1024 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(1024, 10)
FG_INSTANTIATE_ROW(1024, 10)
