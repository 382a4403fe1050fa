// fused_kernel<double, 256> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<double, 256>(const vxg::FusedArgs&, cudaStream_t);
