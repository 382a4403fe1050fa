// fused_kernel<double, 512> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<double, 512>(const vxg::FusedArgs&, cudaStream_t);
