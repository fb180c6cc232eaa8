// One (H_FIRST, U16, INT) instantiation unit of the fused streaming kernel:
// kernel pointers per (HW, VS) bucket and the launcher. Each fused_inst_*.cu
// expands ZG_FUSED_INSTANCE once; the units are separate to compile in
// parallel.
#pragma once

#include "fused_kernel.cuh"

#include <algorithm>

#define ZG_FUSED_INSTANCE(NAME, HF, U16, INT)                                                                      \
	namespace zg {                                                                                                 \
	namespace {                                                                                                    \
	template <int HW, int VS>                                                                                      \
	const void *ptr_##NAME()                                                                                       \
	{                                                                                                              \
		return reinterpret_cast<const void *>(&fused_detail::fused_kernel<HF, U16, HW, VS, INT>);                  \
	}                                                                                                              \
	template <int HW>                                                                                              \
	const void *ptr_vs_##NAME(int vs)                                                                              \
	{                                                                                                              \
		switch (vs) {                                                                                              \
		case 0: return ptr_##NAME<HW, 8>();                                                                        \
		case 1: return ptr_##NAME<HW, 12>();                                                                       \
		case 2: return ptr_##NAME<HW, 16>();                                                                       \
		default: return ptr_##NAME<HW, 24>();                                                                      \
		}                                                                                                          \
	}                                                                                                              \
	}                                                                                                              \
	const void *fused_kernel_ptr_##NAME(int hw, int vs)                                                            \
	{                                                                                                              \
		return hw == 0 ? ptr_vs_##NAME<6>(vs) : (hw == 1 ? ptr_vs_##NAME<8>(vs) : ptr_vs_##NAME<16>(vs));          \
	}                                                                                                              \
	cudaError_t launch_fused_##NAME(int hw, int vs, const FusedJob *jobs, int num_jobs, int total_tiles,          \
	                                const SmemLayout &L, int grid, const FusedJob &single, const WorkChunks &C,    \
	                                cudaStream_t stream)                                                           \
	{                                                                                                              \
		const void *k = fused_kernel_ptr_##NAME(hw, vs);                                                           \
		cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,                      \
		                                     static_cast<int>(fused_max_smem()));                                  \
		if (e != cudaSuccess)                                                                                      \
			return e;                                                                                              \
		FusedJob one = single;                                                                                     \
		SmemLayout layout = L;                                                                                     \
		WorkChunks chunks = C;                                                                                     \
		if (chunks.sched)                                                                                          \
			grid = std::max(1, std::min(grid, chunks.num));                                                        \
		void *args[] = { &jobs, &num_jobs, &total_tiles, &one, &layout, &chunks };                                 \
		return cudaLaunchKernel(k, dim3(grid), dim3(kStreamThreads), args, static_cast<size_t>(L.total_bytes),    \
		                        stream);                                                                           \
	}                                                                                                              \
	}
