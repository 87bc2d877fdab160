// svd_s3.cu — shared-memory form of the Jacobi SVD kernel (svd_kernel.cuh), 7x7 and 8x8 patches.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD_SM(4, 16, 10, true)
PGSVT_INSTANTIATE_SVD_SM(4, 16, 16, true)
PGSVT_INSTANTIATE_SVD_SM(4, 16, 22, true)
