// double instantiation of the fused convolution pass
#define GB_T double
#define GB_CONV_NAME launch_conv_f64
#include "gbfft_conv_launch.inl"
