// complex<double> pipelined power-of-two c2c kernels in double-float arithmetic
#define GB_T double
#define GB_DF 1
#define GB_PIPE_NAME launch_pipe_df64_c2c
#define GB_GROUP 0
#include "gbfft_pipe_launch.inl"
