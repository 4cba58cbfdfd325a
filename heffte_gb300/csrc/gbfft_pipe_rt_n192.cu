// Pipelined complex float kernels compiled for the plan of length 192.
#define GBFFT_RT_LEN 192
#include "gbfft_pipe_rt_launch.inl"
