// svd_i0.cu — instantiations of the Jacobi SVD kernel (svd_kernel.cuh).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(4, 4, 10)
PGSVT_INSTANTIATE_SVD(4, 4, 16)
