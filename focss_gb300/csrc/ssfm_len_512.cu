// ssfm_len_512.cu -- instantiation of the split-step passes for length-512 sub-FFTs.
#include "ssfm_kernels.cuh"
FG_INSTANTIATE_COL(512, 9)
FG_INSTANTIATE_ROW(512, 9)
