// double instantiation of the pipelined power-of-two kernels
#define GB_T double
#define GB_PIPE_NAME launch_pipe_f64
#include "gbfft_pipe_launch.inl"
