// Depth conversion kernel interface (depth_kernel.cu) and zimg's choice of
// conversion (depth.cpp:43-66, quantize.h:19-45), shared by the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace zg {

struct DepthLaunch {
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;
	int width, height;
	float scale, offset;  // mode 2 and 3: x * scale + offset
	float vmax;           // mode 3: 2^depth - 1
	unsigned shift;       // mode 1
	unsigned seq;         // mode 3: plane index (dither table variant)
	int ordered;          // mode 3: ordered dither, else none
	int vec_in, vec_out;  // planes aligned for 8-sample vector loads / stores
};

// in_type / out_type: 0 BYTE, 1 WORD, 2 HALF, 3 FLOAT; mode 1 left shift,
// 2 to FLOAT or HALF, 3 dither to integer.
cudaError_t launch_depth(int in_type, int out_type, int mode, const DepthLaunch &L, cudaStream_t stream);

} // namespace zg
