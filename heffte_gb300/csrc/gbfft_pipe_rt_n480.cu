// Pipelined complex float kernels compiled for the plan of length 480.
#define GBFFT_RT_LEN 480
#include "gbfft_pipe_rt_launch.inl"
