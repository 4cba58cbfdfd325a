// Pipelined complex float kernels compiled for the plan of length 576.
#define GBFFT_RT_LEN 576
#include "gbfft_pipe_rt_launch.inl"
