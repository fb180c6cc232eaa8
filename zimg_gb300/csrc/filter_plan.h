// Host-side planning for one resize pass: zimg's filter kernels, its FP64
// filter matrix and the f32 / int16 tap tables the GPU kernels consume.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace zg {

// Error categories, mapped to zg_error_code at the C boundary (zimg's
// exception hierarchy, src/zimg/common/except.h:13-41).
struct Error : std::runtime_error {
	int code;
	Error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

enum ErrorCode {
	kErrUnknown = -1,
	kErrOutOfMemory = 1,
	kErrUserCallbackFailed = 2,
	kErrLogic = 1 << 10,
	kErrIllegalArgument = 2 << 10,
	kErrEnumOutOfRange = (2 << 10) + 1,
	kErrInvalidImageSize = (2 << 10) + 2,
	kErrUnsupported = 3 << 10,
	kErrUnsupportedSubsampling = (3 << 10) + 1,
	kErrNoColorspaceConversion = (3 << 10) + 2,
	kErrNoFieldParityConversion = (3 << 10) + 3,
	kErrResamplingNotAvailable = (3 << 10) + 4,
	kErrGreyscaleSubsampling = (1 << 10) + 1,
	kErrColorFamilyMismatch = (1 << 10) + 2,
	kErrImageNotDivisible = (1 << 10) + 3,
	kErrBitDepthOverflow = (1 << 10) + 4,
};

// A resampling kernel f(x) with support s (src/zimg/resize/filter.h:14-128).
class Kernel {
public:
	enum Kind { POINT = 0, BILINEAR = 1, BICUBIC = 2, SPLINE16 = 3, SPLINE36 = 4, LANCZOS = 5, SPLINE64 = 6 };

	// param_a / param_b as the API's filter_param_a / filter_param_b, NaN for
	// the library default (zimg.cpp:320-350).
	Kernel(int kind, double param_a, double param_b);

	unsigned support() const { return support_; }
	double operator()(double x) const;
	int kind() const { return kind_; }

private:
	int kind_;
	unsigned support_ = 0;
	unsigned taps_ = 0;
	double p0_ = 0, p2_ = 0, p3_ = 0, q0_ = 0, q1_ = 0, q2_ = 0, q3_ = 0;
};

// The tap tables of one pass (zimg's FilterContext, filter.h:133-165), rows
// packed densely: tap (i, k) of output i is at [i * width + k] and applies to
// input sample left[i] + k.
struct FilterTable {
	unsigned width = 0;       // taps per output
	unsigned rows = 0;        // outputs
	unsigned input_width = 0; // inputs
	std::vector<float> f32;
	std::vector<int16_t> i16;
	std::vector<unsigned> left;
};

// compute_filter (filter.cpp:249-306) followed by matrix_to_filter
// (filter.cpp:43-127).
FilterTable compute_filter(const Kernel &f, unsigned src_dim, unsigned dst_dim, double shift, double width);

// Pass order of ResizeConversion::create (resize.cpp:12-18,38-104).
// Returns the number of passes; order[p] is true for a horizontal pass.
int plan_pass_order(unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h, double shift_w, double shift_h,
                    double subwidth, double subheight, bool order[2]);

} // namespace zg
