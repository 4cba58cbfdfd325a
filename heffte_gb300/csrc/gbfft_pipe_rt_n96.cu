// Pipelined complex float kernels compiled for the plan of length 96.
#define GBFFT_RT_LEN 96
#include "gbfft_pipe_rt_launch.inl"
