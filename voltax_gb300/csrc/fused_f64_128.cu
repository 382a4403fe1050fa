// fused_kernel<double, 128> and its launcher (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused<double, 128>(const vxg::FusedArgs&, cudaStream_t);
