// svd_i6.cu — alternative shapes of the Jacobi SVD kernel for the autotuner
// (more lanes per patch, fewer rows per lane; see svd.cu).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(3, 16, 10)
PGSVT_INSTANTIATE_SVD(3, 16, 16)
PGSVT_INSTANTIATE_SVD(3, 16, 22)
