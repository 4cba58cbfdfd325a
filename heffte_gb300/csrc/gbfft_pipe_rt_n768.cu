// Pipelined complex float kernels compiled for the plan of length 768.
#define GBFFT_RT_LEN 768
#include "gbfft_pipe_rt_launch.inl"
