// Straight-alpha premultiply / unpremultiply of FLOAT planes (alpha_kernel.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace zg {

struct AlphaLaunch {
	void *planes[3];     // colour planes, processed in place
	ptrdiff_t stride;    // bytes, shared by the colour planes
	const void *alpha;
	ptrdiff_t alpha_stride;
	int num_planes;      // 1 (GREY) or 3
	int width, height;
};

// inverse false: x * alpha; true: x / clamp(alpha, 0, 1), 0 where that is 0.
cudaError_t launch_alpha(const AlphaLaunch &L, bool inverse, cudaStream_t stream);

} // namespace zg
