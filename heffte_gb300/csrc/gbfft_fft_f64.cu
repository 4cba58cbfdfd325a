// double instantiation of the batched transform kernels
#define GB_T double
#define GB_LAUNCH_NAME launch_kernel_f64
#include "gbfft_launch.inl"
