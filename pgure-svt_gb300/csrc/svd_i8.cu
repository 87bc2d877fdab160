// svd_i8.cu — 8 rows per lane forms of the Jacobi SVD kernel (svd_kernel.cuh):
// 4x4 patches on 2 lanes, 7x7 and 8x8 patches on 8 lanes.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(8, 2, 10)
PGSVT_INSTANTIATE_SVD(8, 2, 16)
PGSVT_INSTANTIATE_SVD(8, 8, 10)
PGSVT_INSTANTIATE_SVD(8, 8, 16)
