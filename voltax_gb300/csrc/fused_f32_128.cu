// fused_kernel<float, 128> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<float, 128>(const vxg::FusedArgs&, cudaStream_t);
