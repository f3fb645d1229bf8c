#define GB_T float
#define GB_T_IS_FLOAT 1
#include "kernels_impl.cuh"
