// Pipelined complex float kernels compiled for the plan of length 160.
#define GBFFT_RT_LEN 160
#include "gbfft_pipe_rt_launch.inl"
