// Pipelined complex float kernels compiled for the plan of length 448.
#define GBFFT_RT_LEN 448
#include "gbfft_pipe_rt_launch.inl"
