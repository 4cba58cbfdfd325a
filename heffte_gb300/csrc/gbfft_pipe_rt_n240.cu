// Pipelined complex float kernels compiled for the plan of length 240.
#define GBFFT_RT_LEN 240
#include "gbfft_pipe_rt_launch.inl"
