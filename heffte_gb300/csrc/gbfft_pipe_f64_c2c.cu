// double instantiation of the pipelined power-of-two kernels (c2c group)
#define GB_T double
#define GB_PIPE_NAME launch_pipe_f64_c2c
#define GB_GROUP 0
#include "gbfft_pipe_launch.inl"
