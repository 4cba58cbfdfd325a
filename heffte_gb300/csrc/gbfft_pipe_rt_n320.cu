// Pipelined complex float kernels compiled for the plan of length 320.
#define GBFFT_RT_LEN 320
#include "gbfft_pipe_rt_launch.inl"
