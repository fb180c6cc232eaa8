// Launch interface between the host planner and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace zg {

// Device-resident tap tables of one pass (the GPU copy of a FilterTable).
//   left[i]            first input sample of output i
//   f32[i*width + k]   float taps
//   i16[i*width + k]   signed 1.14 taps
//   bias[i]            -32768 * sum_k i16[i*width+k] (mod 2^32): folds zimg's
//                      "x - 32768" unpacking (resize_impl.cpp:31-34) into one
//                      constant so the inner loop is a plain multiply-add.
struct PassTables {
	const unsigned *left;
	const float *f32;
	const int16_t *i16;
	const int32_t *bias;
	unsigned width;        // taps per output
	unsigned rows;         // outputs along the filtered axis
	unsigned input_width;  // inputs along the filtered axis
};

enum class Sample { U16, F32 };

// One pass over a whole plane. For a horizontal pass the plane has
// `lines` rows of input_width samples -> rows outputs each; for a vertical
// pass it has `lines` columns, input_width rows -> rows rows.
struct PassLaunch {
	PassTables t;
	bool horizontal;
	Sample sample;
	int32_t pixel_max;     // (1 << depth) - 1 for U16
	unsigned lines;        // height (H) or width (V) of the plane
	const void *src;
	ptrdiff_t src_stride;  // bytes
	void *dst;
	ptrdiff_t dst_stride;  // bytes
};

cudaError_t launch_pass(const PassLaunch &l, cudaStream_t stream);

} // namespace zg
