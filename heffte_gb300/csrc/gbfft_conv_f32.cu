// float instantiation of the fused convolution pass
#define GB_T float
#define GB_CONV_NAME launch_conv_f32
#include "gbfft_conv_launch.inl"
