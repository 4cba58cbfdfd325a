// Pipelined complex float kernels compiled for the plan of length 720.
#define GBFFT_RT_LEN 720
#include "gbfft_pipe_rt_launch.inl"
