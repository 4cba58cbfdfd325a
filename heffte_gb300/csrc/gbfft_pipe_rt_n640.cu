// Pipelined complex float kernels compiled for the plan of length 640.
#define GBFFT_RT_LEN 640
#include "gbfft_pipe_rt_launch.inl"
