// float instantiation of the batched transform kernels
#define GB_T float
#define GB_LAUNCH_NAME launch_kernel_f32
#include "gbfft_launch.inl"
