// fused_kernel<double, 64> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<double, 64>(const vxg::FusedArgs&, cudaStream_t);
