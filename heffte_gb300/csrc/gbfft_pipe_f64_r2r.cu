// double instantiation of the pipelined power-of-two kernels (r2r group)
#define GB_T double
#define GB_PIPE_NAME launch_pipe_f64_r2r
#define GB_GROUP 2
#include "gbfft_pipe_launch.inl"
