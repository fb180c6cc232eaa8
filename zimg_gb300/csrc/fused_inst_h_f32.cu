// Instantiations of the fused tile kernel for H_FIRST=true, U16=false.
#include "fused_kernel.cuh"

namespace zg {

namespace {

template <int HW, int VS>
const void *ptr()
{
	return reinterpret_cast<const void *>(&fused_detail::fused_kernel<true, false, HW, VS>);
}

template <int HW>
const void *ptr_vs(int vs)
{
	switch (vs) {
	case 0: return ptr<HW, 8>();
	case 1: return ptr<HW, 12>();
	case 2: return ptr<HW, 16>();
	default: return ptr<HW, 24>();
	}
}

} // namespace

const void *fused_kernel_ptr_h_f32(int hw, int vs)
{
	return hw == 0 ? ptr_vs<6>(vs) : (hw == 1 ? ptr_vs<8>(vs) : ptr_vs<16>(vs));
}

cudaError_t launch_fused_h_f32(int hw, int vs, const FusedJob *jobs, int num_jobs, int total_tiles, const SmemLayout &L,
                            int grid, const FusedJob &single, cudaStream_t stream)
{
	const void *k = fused_kernel_ptr_h_f32(hw, vs);
	cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(fused_max_smem()));
	if (e != cudaSuccess)
		return e;
	FusedJob one = single;
	SmemLayout layout = L;
	void *args[] = { &jobs, &num_jobs, &total_tiles, &one, &layout };
	return cudaLaunchKernel(k, dim3(grid), dim3(kStreamThreads), args, static_cast<size_t>(L.total_bytes), stream);
}

} // namespace zg
