// fused_kernel<float, 64> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<float, 64>(const vxg::FusedArgs&, cudaStream_t);
