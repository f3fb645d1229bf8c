#define GB_T float
#include "kernels_impl.cuh"
