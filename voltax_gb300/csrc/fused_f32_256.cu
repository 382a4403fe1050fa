// fused_kernel<float, 256> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<float, 256>(const vxg::FusedArgs&, cudaStream_t);
