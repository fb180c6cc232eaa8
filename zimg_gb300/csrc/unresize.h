// Unresize (zimg's src/zimg/unresize/): the least-squares inverse of a
// bilinear upsampling, FP32. Host context construction (unresize_plan.cpp)
// and the device passes (unresize_kernel.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

namespace zg {

// One axis: `up` input samples -> `orig` output samples.
struct UnresizeContext {
	unsigned up = 0, orig = 0;
	unsigned row_size = 0;
	std::vector<float> coef;        // [orig][row_size]: row r of A', from offset[r]
	std::vector<unsigned> offset;   // [orig]
	std::vector<float> lu_c, lu_l, lu_u;  // tridiagonal LU of A'A (lu_l inverted)
};

// Returns false when orig > up (zimg: "unresize can not upscale").
bool build_unresize_context(unsigned orig, unsigned up, double shift, UnresizeContext *out);

// Zimg's pass order (unresize.cpp:14-19).
bool unresize_h_first(double xscale, double yscale);

// Device copy of a context.
struct UnresizeTables {
	const float *coef;
	const unsigned *offset;
	const float *lu_c, *lu_l, *lu_u;
	unsigned up, orig, row_size;
};

// One pass over a FLOAT plane: horizontal (lines of `up` -> `orig` samples,
// `lines` of them) or vertical (`cols` columns of `up` lines -> `orig` lines).
cudaError_t launch_unresize(const UnresizeTables &t, bool horizontal, unsigned lines_or_cols, const void *src,
                            ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, cudaStream_t stream);

} // namespace zg
