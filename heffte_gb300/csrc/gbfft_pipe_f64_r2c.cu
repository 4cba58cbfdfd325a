// double instantiation of the pipelined power-of-two kernels (r2c group)
#define GB_T double
#define GB_PIPE_NAME launch_pipe_f64_r2c
#define GB_GROUP 1
#include "gbfft_pipe_launch.inl"
