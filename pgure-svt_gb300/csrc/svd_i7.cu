// svd_i7.cu — alternative shapes of the Jacobi SVD kernel for the autotuner
// (one patch per warp for 7x7 and 8x8 patches; see svd.cu).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(2, 32, 10)
PGSVT_INSTANTIATE_SVD(2, 32, 16)
PGSVT_INSTANTIATE_SVD(2, 32, 22)
