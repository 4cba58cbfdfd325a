// Pipelined complex float kernels compiled for the plan of length 384.
#define GBFFT_RT_LEN 384
#include "gbfft_pipe_rt_launch.inl"
