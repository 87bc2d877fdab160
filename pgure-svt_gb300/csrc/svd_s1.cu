// svd_s1.cu — shared-memory form of the Jacobi SVD kernel (svd_kernel.cuh), 5x5 patches.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD_SM(4, 8, 10, true)
PGSVT_INSTANTIATE_SVD_SM(4, 8, 16, true)
PGSVT_INSTANTIATE_SVD_SM(4, 8, 22, true)
