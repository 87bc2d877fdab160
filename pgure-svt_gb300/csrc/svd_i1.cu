// svd_i1.cu — instantiations of the Jacobi SVD kernel (svd_kernel.cuh).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(4, 8, 10)
PGSVT_INSTANTIATE_SVD(4, 8, 16)
PGSVT_INSTANTIATE_SVD(4, 8, 22)
