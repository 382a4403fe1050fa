// fused_warp_kernel<float, 2/4/8> and their launchers (see fused.cuh).
#include "fused.cuh"

template int vxg::launch_fused_warp<float, 2>(const vxg::FusedArgs&, cudaStream_t);
template int vxg::launch_fused_warp<float, 4>(const vxg::FusedArgs&, cudaStream_t);
template int vxg::launch_fused_warp<float, 8>(const vxg::FusedArgs&, cudaStream_t);
