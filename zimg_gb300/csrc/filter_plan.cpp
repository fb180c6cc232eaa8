// Filter-table planning on the host, in FP64, exactly as zimg computes it.
// Compiled with -ffp-contract=off so every product and sum is rounded the way
// zimg's own build rounds it.
#include "filter_plan.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>

namespace zg {

namespace {

constexpr double kPi = 3.14159265358979323846;

// sinc with zimg's guard for x == 0 (filter.cpp:21-25). sin comes from libm,
// as zimg_x_sin does by default (libm_wrapper.cpp:10).
double sinc(double x)
{
	return x == 0.0 ? 1.0 : std::sin(x * kPi) / (x * kPi);
}

// Horner form c0 + x(c1 + x(c2 + x c3)) (filter.cpp:27-30).
double horner3(double x, double c0, double c1, double c2, double c3)
{
	return c0 + x * (c1 + x * (c2 + x * c3));
}

// Rounding that keeps round(x - 1) == round(x) - 1 on the pixel grid
// (filter.cpp:32-40).
double grid_round(double x)
{
	return x < 0 ? std::floor(x + 0.5) : std::floor(x + 0.49999999999999994);
}

// One row of the FP64 filter matrix. zimg stores each row as one contiguous
// run that only grows when a write changes the stored value
// (matrix.cpp:14-21,103-129); the run's extent defines filter_width and left,
// so that rule is reproduced here over a dense scratch line.
class BandRow {
public:
	explicit BandRow(std::vector<double> &line) : line_(line) {}

	double get(size_t j) const { return (used_ && j >= lo_ && j < hi_) ? line_[j] : 0.0; }

	void set(size_t j, double v)
	{
		if (get(j) == v)
			return;
		if (!used_) {
			lo_ = j;
			hi_ = j + 1;
			used_ = true;
		} else {
			lo_ = std::min(lo_, j);
			hi_ = std::max(hi_, j + 1);
		}
		line_[j] = v;
	}

	size_t lo() const { return lo_; }
	size_t hi() const { return hi_; }

	// Copy the run out and zero the scratch line for the next row.
	std::vector<double> take()
	{
		std::vector<double> run(line_.begin() + lo_, line_.begin() + hi_);
		std::fill(line_.begin() + lo_, line_.begin() + hi_, 0.0);
		return run;
	}

private:
	std::vector<double> &line_;
	size_t lo_ = 0, hi_ = 0;
	bool used_ = false;
};

} // namespace


Kernel::Kernel(int kind, double a, double b) : kind_(kind)
{
	switch (kind) {
	case POINT: support_ = 0; break;
	case BILINEAR: support_ = 1; break;
	case BICUBIC: {
		// Mitchell-Netravali (b, c) cubic; defaults b=0, c=0.5 (filter.h:58-60,
		// filter.cpp:147-155).
		double B = std::isnan(a) ? 0.0 : a;
		double C = std::isnan(b) ? 0.5 : b;
		p0_ = (6.0 - 2.0 * B) / 6.0;
		p2_ = (-18.0 + 12.0 * B + 6.0 * C) / 6.0;
		p3_ = (12.0 - 9.0 * B - 6.0 * C) / 6.0;
		q0_ = (8.0 * B + 24.0 * C) / 6.0;
		q1_ = (-12.0 * B - 48.0 * C) / 6.0;
		q2_ = (6.0 * B + 30.0 * C) / 6.0;
		q3_ = (-B - 6.0 * C) / 6.0;
		support_ = 2;
		break;
	}
	case SPLINE16: support_ = 2; break;
	case SPLINE36: support_ = 3; break;
	case SPLINE64: support_ = 4; break;
	case LANCZOS: {
		// NaN -> 3 taps; otherwise clamped to [1, UINT_MAX] and truncated
		// (zimg.cpp:343-345); 16 or more taps is illegal (filter.cpp:232-238).
		double t = std::isnan(a) ? 3.0 : std::clamp(a, 1.0, static_cast<double>(UINT_MAX));
		taps_ = static_cast<unsigned>(t);
		if (taps_ >= 16)
			throw Error(kErrIllegalArgument, "lanczos tap count too high");
		support_ = taps_;
		break;
	}
	default:
		throw Error(kErrEnumOutOfRange, "unrecognized resampling filter");
	}
}

double Kernel::operator()(double x) const
{
	// Piecewise kernels of filter.cpp:136-246; spline coefficients are the
	// published AviSynth Spline16/36/64 polynomials.
	switch (kind_) {
	case POINT:
		return 1.0;
	case BILINEAR:
		return std::max(1.0 - std::abs(x), 0.0);
	case BICUBIC:
		x = std::abs(x);
		if (x < 1.0) return horner3(x, p0_, 0.0, p2_, p3_);
		if (x < 2.0) return horner3(x, q0_, q1_, q2_, q3_);
		return 0.0;
	case SPLINE16:
		x = std::abs(x);
		if (x < 1.0) return horner3(x, 1.0, -1.0 / 5.0, -9.0 / 5.0, 1.0);
		if (x < 2.0) return horner3(x - 1.0, 0.0, -7.0 / 15.0, 4.0 / 5.0, -1.0 / 3.0);
		return 0.0;
	case SPLINE36:
		x = std::abs(x);
		if (x < 1.0) return horner3(x, 1.0, -3.0 / 209.0, -453.0 / 209.0, 13.0 / 11.0);
		if (x < 2.0) return horner3(x - 1.0, 0.0, -156.0 / 209.0, 270.0 / 209.0, -6.0 / 11.0);
		if (x < 3.0) return horner3(x - 2.0, 0.0, 26.0 / 209.0, -45.0 / 209.0, 1.0 / 11.0);
		return 0.0;
	case SPLINE64:
		x = std::abs(x);
		if (x < 1.0) return horner3(x, 1.0, -3.0 / 2911.0, -6387.0 / 2911.0, 49.0 / 41.0);
		if (x < 2.0) return horner3(x - 1.0, 0.0, -2328.0 / 2911.0, 4032.0 / 2911.0, -24.0 / 41.0);
		if (x < 3.0) return horner3(x - 2.0, 0.0, 582.0 / 2911.0, -1008.0 / 2911.0, 6.0 / 41.0);
		if (x < 4.0) return horner3(x - 3.0, 0.0, -97.0 / 2911.0, 168.0 / 2911.0, -1.0 / 41.0);
		return 0.0;
	case LANCZOS:
		x = std::abs(x);
		return x < taps_ ? sinc(x) * sinc(x / taps_) : 0.0;
	default:
		return 0.0;
	}
}


FilterTable compute_filter(const Kernel &f, unsigned src_dim, unsigned dst_dim, double shift, double width)
{
	if (!src_dim || !dst_dim)
		throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");

	// Geometry of the resampling (filter.cpp:251-257).
	const double scale = static_cast<double>(dst_dim) / width;
	const double step = std::min(scale, 1.0);
	const double support = static_cast<double>(f.support()) / step;
	const unsigned window = std::max(static_cast<unsigned>(std::ceil(support)) * 2U, 1U);
	if (support > static_cast<unsigned>(UINT_MAX / 2))
		throw Error(kErrResamplingNotAvailable, "filter width too great");

	std::vector<double> line(src_dim, 0.0);
	std::vector<std::vector<double>> runs(dst_dim);
	std::vector<size_t> run_lo(dst_dim), run_hi(dst_dim);
	const double last_valid = std::nextafter(static_cast<double>(src_dim), -INFINITY);

	for (unsigned i = 0; i < dst_dim; ++i) {
		BandRow row(line);

		// Output sample i sits at pos on the input grid; its window starts at
		// the grid-rounded pos - window/2 (filter.cpp:262-264).
		const double pos = (i + 0.5) / scale + shift;
		const double first = grid_round(pos - window / 2.0) + 0.5;

		double total = 0.0;
		for (unsigned j = 0; j < window; ++j)
			total += f((first + j - pos) * step);

		// Normalised taps; positions outside the image mirror about its edges,
		// then clamp, and taps landing on one sample add up (filter.cpp:272-291).
		size_t min_idx = SIZE_MAX;
		for (unsigned j = 0; j < window; ++j) {
			const double xpos = first + j;
			double p = xpos < 0.0 ? -xpos : (xpos >= src_dim ? 2.0 * src_dim - xpos : xpos);
			p = std::clamp(p, 0.0, last_valid);
			const size_t idx = static_cast<size_t>(std::floor(p));
			row.set(idx, row.get(idx) + f((xpos - pos) * step) / total);
			min_idx = std::min(min_idx, idx);
		}

		// Keep an entry at the leftmost index so the left table stays sorted
		// (filter.cpp:294-298).
		if (row.get(min_idx) == 0.0) {
			row.set(min_idx, DBL_EPSILON);
			row.set(min_idx, 0.0);
		}

		run_lo[i] = row.lo();
		run_hi[i] = row.hi();
		runs[i] = row.take();
	}

	// Quantise (filter.cpp:43-127): one common width, left clamped so the
	// window stays inside the input, taps rounded with error diffusion, and the
	// int16 row forced to sum to exactly 1 << 14 on its largest tap.
	size_t width_taps = 0;
	for (unsigned i = 0; i < dst_dim; ++i)
		width_taps = std::max(width_taps, run_hi[i] - run_lo[i]);

	FilterTable t;
	t.width = static_cast<unsigned>(width_taps);
	t.rows = dst_dim;
	t.input_width = src_dim;
	t.f32.assign(static_cast<size_t>(t.width) * t.rows, 0.0f);
	t.i16.assign(static_cast<size_t>(t.width) * t.rows, 0);
	t.left.assign(t.rows, 0);

	for (unsigned i = 0; i < dst_dim; ++i) {
		const size_t left = std::min(run_lo[i], static_cast<size_t>(src_dim) - width_taps);
		double carry_f32 = 0.0;
		double carry_i16 = 0.0;
		int16_t sum_i16 = 0;
		int16_t biggest = 0;
		size_t biggest_at = 0;

		float *out_f = &t.f32[static_cast<size_t>(i) * t.width];
		int16_t *out_q = &t.i16[static_cast<size_t>(i) * t.width];
		for (size_t k = 0; k < width_taps; ++k) {
			const size_t col = left + k;
			const double c = (col >= run_lo[i] && col < run_hi[i]) ? runs[i][col - run_lo[i]] : 0.0;

			const double want_f = c - carry_f32;
			const double want_q = c * (1 << 14) - carry_i16;
			const float got_f = static_cast<float>(want_f);
			const int16_t got_q = static_cast<int16_t>(std::lrint(want_q));
			carry_f32 = static_cast<double>(got_f) - want_f;
			carry_i16 = static_cast<double>(got_q) - want_q;

			if (std::abs(got_q) > std::abs(biggest)) {
				biggest = got_q;
				biggest_at = k;
			}
			sum_i16 = static_cast<int16_t>(sum_i16 + got_q);
			out_f[k] = got_f;
			out_q[k] = got_q;
		}
		out_q[biggest_at] = static_cast<int16_t>(out_q[biggest_at] + ((1 << 14) - sum_i16));
		t.left[i] = static_cast<unsigned>(left);
	}
	return t;
}


int plan_pass_order(unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h, double shift_w, double shift_h,
                    double subwidth, double subheight, bool order[2])
{
	const bool skip_h = src_w == dst_w && shift_w == 0 && subwidth == src_w;
	const bool skip_v = src_h == dst_h && shift_h == 0 && subheight == src_h;
	if (skip_h && skip_v)
		return 0;
	if (skip_h) {
		order[0] = false;
		return 1;
	}
	if (skip_v) {
		order[0] = true;
		return 1;
	}
	// Relative line-buffer cost of the two orders (resize.cpp:12-18).
	const double xs = static_cast<double>(dst_w) / subwidth;
	const double ys = static_cast<double>(dst_h) / subheight;
	const double h_cost = std::max(xs, 1.0) * 2.0 + xs * std::max(ys, 1.0);
	const double v_cost = std::max(ys, 1.0) + ys * std::max(xs, 1.0) * 2.0;
	const bool h_first = h_cost < v_cost;
	order[0] = h_first;
	order[1] = !h_first;
	return 2;
}

} // namespace zg
