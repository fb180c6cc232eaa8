// zimg's simple graph filters on device planes (alpha_kernel.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

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

// Every sample of a plane set to `value` (its low `bytes` bytes; bytes 1, 2
// or 4).
cudaError_t launch_fill(void *dst, ptrdiff_t stride, int width, int height, int bytes, uint32_t value,
                        cudaStream_t stream);

} // namespace zg
