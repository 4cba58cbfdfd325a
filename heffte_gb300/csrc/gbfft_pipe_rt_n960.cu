// Pipelined complex float kernels compiled for the plan of length 960.
#define GBFFT_RT_LEN 960
#include "gbfft_pipe_rt_launch.inl"
