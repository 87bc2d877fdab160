// svd_s2.cu — shared-memory form of the Jacobi SVD kernel (svd_kernel.cuh), 6x6 patches.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD_SM(5, 8, 10, true)
PGSVT_INSTANTIATE_SVD_SM(5, 8, 16, true)
PGSVT_INSTANTIATE_SVD_SM(5, 8, 22, true)
