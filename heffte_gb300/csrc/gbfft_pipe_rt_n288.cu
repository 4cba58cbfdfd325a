// Pipelined complex float kernels compiled for the plan of length 288.
#define GBFFT_RT_LEN 288
#include "gbfft_pipe_rt_launch.inl"
