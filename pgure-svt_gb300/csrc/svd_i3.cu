// svd_i3.cu — instantiations of the Jacobi SVD kernel (svd_kernel.cuh).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(4, 16, 10)
PGSVT_INSTANTIATE_SVD(4, 16, 16)
