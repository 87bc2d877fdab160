// svd_s0.cu — shared-memory form of the Jacobi SVD kernel (svd_kernel.cuh), 2x2..4x4 patches.
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD_SM(4, 4, 10, true)
PGSVT_INSTANTIATE_SVD_SM(4, 4, 16, true)
