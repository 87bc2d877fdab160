// svd_s4.cu — Jacobi SVD kernel (svd_kernel.cuh) for 9x9 to 16x16 patches:
// 8 rows x 32 lanes per patch, columns in shared memory.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD_SM(8, 32, 10, true)
PGSVT_INSTANTIATE_SVD_SM(8, 32, 16, true)
PGSVT_INSTANTIATE_SVD_SM(8, 32, 22, true)
