#define GB_T double
#include "kernels_impl.cuh"
