// ssfm_len_64.cu -- instantiation of the split-step passes for length-64 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(64, 6)
FG_INSTANTIATE_ROW(64, 6)
