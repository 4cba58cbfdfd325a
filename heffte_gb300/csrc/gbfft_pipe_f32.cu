// float instantiation of the pipelined power-of-two kernels
#define GB_T float
#define GB_PIPE_NAME launch_pipe_f32
#include "gbfft_pipe_launch.inl"
