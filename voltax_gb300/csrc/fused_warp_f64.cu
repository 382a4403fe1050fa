// fused_warp_kernel<double, 2/4/8> and their launchers (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused_warp<double, 2>(const vxg::FusedArgs&, cudaStream_t);
template int vxg::launch_fused_warp<double, 4>(const vxg::FusedArgs&, cudaStream_t);
template int vxg::launch_fused_warp<double, 8>(const vxg::FusedArgs&, cudaStream_t);
