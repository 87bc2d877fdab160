// svd_i5.cu — alternative shapes of the Jacobi SVD kernel for the autotuner
// (more lanes per patch, fewer rows per lane; see svd.cu).
#include "svd_kernel.cuh"

PGSVT_INSTANTIATE_SVD(2, 8, 10)
PGSVT_INSTANTIATE_SVD(2, 8, 16)
