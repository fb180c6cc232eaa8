/*
 * C-callable driver around zimg's own resize code, compiled from the reference
 * checkout (never copied into this repository) by oracle/Makefile.
 *
 * This is test infrastructure: it lets the tests, the golden-fixture script and
 * the CPU baseline run the reference's FilterContext construction
 * (src/zimg/resize/filter.cpp:249-306) and its resize filters
 * (src/zimg/resize/resize_impl.cpp:117-267, ISA kernels under
 * src/zimg/resize/{x86,arm}/) on whole planes, the way graphengine would drive
 * them line by line (src/zimg/resize/resize_impl.cpp:130-160).
 */
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <utility>
#include <vector>

#include "common/cpuinfo.h"
#include "common/except.h"
#include "common/pixel.h"
#include "graphengine/filter.h"
#include "colorspace/colorspace.h"
#include "depth/blue.h"
#include "depth/depth.h"
#include "unresize/unresize.h"
#include "resize/filter.h"
#include "resize/resize.h"
#include "resize/resize_impl.h"

namespace {

using zimg::CPUClass;
using zimg::PixelType;

std::unique_ptr<zimg::resize::Filter> make_filter(int kind, double a, double b)
{
	/* Filter enum values and NaN defaults follow zimg.h:374-382 and
	 * zimg.cpp:320-350 (translate_resize_filter). */
	switch (kind) {
	case 0: return std::make_unique<zimg::resize::PointFilter>();
	case 1: return std::make_unique<zimg::resize::BilinearFilter>();
	case 2:
		return std::make_unique<zimg::resize::BicubicFilter>(std::isnan(a) ? 0.0 : a, std::isnan(b) ? 0.5 : b);
	case 3: return std::make_unique<zimg::resize::Spline16Filter>();
	case 4: return std::make_unique<zimg::resize::Spline36Filter>();
	case 6: return std::make_unique<zimg::resize::Spline64Filter>();
	case 5: {
		double t = std::isnan(a) ? 3.0 : std::clamp(a, 1.0, 4294967295.0);
		return std::make_unique<zimg::resize::LanczosFilter>(static_cast<unsigned>(t));
	}
	default:
		throw zimg::error::EnumOutOfRange{ "unrecognized resampling filter" };
	}
}

CPUClass make_cpu(int cpu)
{
	if (cpu == 1) return CPUClass::AUTO;
	if (cpu == 2) return CPUClass::AUTO_64B;
	return CPUClass::NONE;
}

void set_err(char *err, size_t errlen, const char *msg)
{
	if (err && errlen) {
		std::strncpy(err, msg, errlen - 1);
		err[errlen - 1] = '\0';
	}
}

int catch_all(char *err, size_t errlen)
{
	try {
		throw;
	} catch (const zimg::error::Exception &e) {
		set_err(err, errlen, e.what());
		return 1;
	} catch (const std::exception &e) {
		set_err(err, errlen, e.what());
		return 2;
	}
}

struct Plan {
	std::unique_ptr<zimg::resize::Filter> kernel;
	std::unique_ptr<graphengine::Filter> first;
	std::unique_ptr<graphengine::Filter> second;
	unsigned src_w, src_h, dst_w, dst_h, bytes;
};

void *aligned_buf(size_t size)
{
	size = (size + 63) & ~static_cast<size_t>(63);
	return std::aligned_alloc(64, size ? size : 64);
}

/* Run one filter over an entire plane: every output line, full width. */
void run_filter(const graphengine::Filter &f, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	const graphengine::FilterDescriptor &desc = f.descriptor();
	graphengine::BufferDescriptor in{ const_cast<void *>(src), src_stride, ~0U };
	graphengine::BufferDescriptor out{ dst, dst_stride, ~0U };

	void *ctx = desc.context_size ? aligned_buf(desc.context_size) : nullptr;
	void *tmp = desc.scratchpad_size ? aligned_buf(desc.scratchpad_size) : nullptr;
	if ((desc.context_size && !ctx) || (desc.scratchpad_size && !tmp)) {
		std::free(ctx);
		std::free(tmp);
		throw std::bad_alloc{};
	}
	if (ctx)
		f.init_context(ctx);

	unsigned step = desc.step ? desc.step : 1;
	for (unsigned i = 0; i < desc.format.height; i += step)
		f.process(&in, &out, i, 0, desc.format.width, ctx, tmp);

	std::free(ctx);
	std::free(tmp);
}

// Whole planes through a filter of three planes (a colorspace conversion).
void run_filter3(const graphengine::Filter &f, const void *const src[3], const ptrdiff_t src_stride[3],
                 void *const dst[3], const ptrdiff_t dst_stride[3])
{
	const graphengine::FilterDescriptor &desc = f.descriptor();
	graphengine::BufferDescriptor in[3], out[3];
	for (int p = 0; p < 3; ++p) {
		in[p] = graphengine::BufferDescriptor{ const_cast<void *>(src[p]), src_stride[p], ~0U };
		out[p] = graphengine::BufferDescriptor{ dst[p], dst_stride[p], ~0U };
	}
	void *tmp = desc.scratchpad_size ? aligned_buf(desc.scratchpad_size) : nullptr;
	if (desc.scratchpad_size && !tmp)
		throw std::bad_alloc{};
	for (unsigned i = 0; i < desc.format.height; ++i)
		f.process(in, out, i, 0, desc.format.width, nullptr, tmp);
	std::free(tmp);
}

} // namespace


extern "C" {

/* Evaluate a filter kernel f(x) at n points; returns the support in *support. */
int ref_filter_eval(int kind, double a, double b, const double *x, double *y, size_t n, unsigned *support, char *err, size_t errlen)
{
	try {
		auto f = make_filter(kind, a, b);
		for (size_t i = 0; i < n; ++i)
			y[i] = (*f)(x[i]);
		if (support)
			*support = f->support();
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

/*
 * compute_filter (filter.cpp:249-306). First call with data == nullptr to get
 * the shape; then call again with data_f32[rows*width], data_i16[rows*width]
 * and left[rows] (rows packed densely, without the reference's stride padding).
 */
int ref_compute_filter(int kind, double a, double b, unsigned src_dim, unsigned dst_dim, double shift, double width,
                       unsigned *filter_width, unsigned *filter_rows, unsigned *input_width,
                       float *data_f32, int16_t *data_i16, unsigned *left, char *err, size_t errlen)
{
	try {
		auto f = make_filter(kind, a, b);
		zimg::resize::FilterContext ctx = zimg::resize::compute_filter(*f, src_dim, dst_dim, shift, width);
		*filter_width = ctx.filter_width;
		*filter_rows = ctx.filter_rows;
		*input_width = ctx.input_width;
		if (data_f32) {
			for (unsigned i = 0; i < ctx.filter_rows; ++i) {
				for (unsigned k = 0; k < ctx.filter_width; ++k) {
					data_f32[static_cast<size_t>(i) * ctx.filter_width + k] = ctx.data[static_cast<size_t>(i) * ctx.stride + k];
					data_i16[static_cast<size_t>(i) * ctx.filter_width + k] = ctx.data_i16[static_cast<size_t>(i) * ctx.stride_i16 + k];
				}
				left[i] = ctx.left[i];
			}
		}
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

/* ResizeConversion (resize.cpp:38-104): zero, one or two passes. */
void *ref_plan_create(int pixel_type, unsigned depth, int kind, double a, double b,
                      unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h,
                      double shift_w, double shift_h, double subwidth, double subheight,
                      int cpu, char *err, size_t errlen)
{
	try {
		auto plan = std::make_unique<Plan>();
		plan->kernel = make_filter(kind, a, b);
		PixelType type = static_cast<PixelType>(pixel_type);
		auto pair = zimg::resize::ResizeConversion{ src_w, src_h, type }
			.set_depth(depth)
			.set_filter(plan->kernel.get())
			.set_dst_width(dst_w)
			.set_dst_height(dst_h)
			.set_shift_w(shift_w)
			.set_shift_h(shift_h)
			.set_subwidth(subwidth)
			.set_subheight(subheight)
			.set_cpu(make_cpu(cpu))
			.create();
		plan->first = std::move(pair.first);
		plan->second = std::move(pair.second);
		plan->src_w = src_w;
		plan->src_h = src_h;
		plan->dst_w = dst_w;
		plan->dst_h = dst_h;
		plan->bytes = zimg::pixel_size(type);
		return plan.release();
	} catch (...) {
		catch_all(err, errlen);
		return nullptr;
	}
}

/* One pass built by ResizeImplBuilder (resize_impl.cpp:245-267). */
void *ref_pass_create(int horizontal, unsigned src_w, unsigned src_h, int pixel_type, unsigned depth,
                      unsigned dst_dim, int kind, double a, double b, double shift, double subwidth,
                      int cpu, char *err, size_t errlen)
{
	try {
		auto plan = std::make_unique<Plan>();
		plan->kernel = make_filter(kind, a, b);
		PixelType type = static_cast<PixelType>(pixel_type);
		plan->first = zimg::resize::ResizeImplBuilder{ src_w, src_h, type }
			.set_horizontal(!!horizontal)
			.set_dst_dim(dst_dim)
			.set_depth(depth)
			.set_filter(plan->kernel.get())
			.set_shift(shift)
			.set_subwidth(subwidth)
			.set_cpu(make_cpu(cpu))
			.create();
		plan->src_w = src_w;
		plan->src_h = src_h;
		plan->dst_w = horizontal ? dst_dim : src_w;
		plan->dst_h = horizontal ? src_h : dst_dim;
		plan->bytes = zimg::pixel_size(type);
		return plan.release();
	} catch (...) {
		catch_all(err, errlen);
		return nullptr;
	}
}

void ref_plan_free(void *p)
{
	delete static_cast<Plan *>(p);
}

/* Number of filters in the plan: 0 (copy), 1 or 2. */
int ref_plan_num_passes(const void *p)
{
	const Plan *plan = static_cast<const Plan *>(p);
	return (plan->first ? 1 : 0) + (plan->second ? 1 : 0);
}

/*
 * Run the plan on one whole plane. Thread-safe for concurrent calls on the same
 * plan (filters are immutable; scratch is per call), as zimg's graphs are.
 */
int ref_plan_run(const void *p, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, char *err, size_t errlen)
{
	try {
		const Plan *plan = static_cast<const Plan *>(p);
		if (!plan->first) {
			for (unsigned i = 0; i < plan->dst_h; ++i)
				std::memcpy(static_cast<char *>(dst) + i * dst_stride, static_cast<const char *>(src) + i * src_stride,
				            static_cast<size_t>(plan->dst_w) * plan->bytes);
			return 0;
		}
		if (!plan->second) {
			run_filter(*plan->first, src, src_stride, dst, dst_stride);
			return 0;
		}
		const graphengine::FilterDescriptor &d = plan->first->descriptor();
		ptrdiff_t tmp_stride = (static_cast<ptrdiff_t>(d.format.width) * d.format.bytes_per_sample + 63) & ~static_cast<ptrdiff_t>(63);
		void *tmp = aligned_buf(static_cast<size_t>(tmp_stride) * (d.format.height + 1));
		if (!tmp)
			throw std::bad_alloc{};
		run_filter(*plan->first, src, src_stride, tmp, tmp_stride);
		run_filter(*plan->second, tmp, tmp_stride, dst, dst_stride);
		std::free(tmp);
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

/*
 * zimg's ColorspaceConversion (src/zimg/colorspace/colorspace.h:117-132) on
 * three FLOAT planes. Colorspaces as zimg's internal enum values
 * (colorspace.h:19-60); cpu as ref_plan_create. Returns 3 when the
 * conversion is the identity (no filter; dst untouched).
 */
int ref_colorspace(int m_in, int t_in, int p_in, int m_out, int t_out, int p_out, double peak, int approx, int scene,
                   int adapt, int cpu, unsigned w, unsigned h, const void *const src[3], const ptrdiff_t src_stride[3],
                   void *const dst[3], const ptrdiff_t dst_stride[3], char *err, size_t errlen)
{
	try {
		namespace cs = zimg::colorspace;
		cs::ColorspaceConversion conv{ w, h };
		conv.set_csp_in({ static_cast<cs::MatrixCoefficients>(m_in), static_cast<cs::TransferCharacteristics>(t_in),
		                  static_cast<cs::ColorPrimaries>(p_in) })
			.set_csp_out({ static_cast<cs::MatrixCoefficients>(m_out), static_cast<cs::TransferCharacteristics>(t_out),
			               static_cast<cs::ColorPrimaries>(p_out) })
			.set_peak_luminance(peak)
			.set_approximate_gamma(approx != 0)
			.set_scene_referred(scene != 0)
			.set_chromatic_adaptation(adapt != 0)
			.set_cpu(make_cpu(cpu));
		std::unique_ptr<graphengine::Filter> f = conv.create();
		if (!f)
			return 3;
		run_filter3(*f, src, src_stride, dst, dst_stride);
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

/*
 * zimg's 64 x 64 blue-noise matrix behind RANDOM dither
 * (src/zimg/depth/blue.h:10-13), row-major, into out[4096].
 */
void ref_blue_noise_table(uint8_t *out)
{
	std::memcpy(out, &zimg::depth::blue_noise_table[0][0],
	            zimg::depth::BLUE_NOISE_LEN * zimg::depth::BLUE_NOISE_LEN);
}

/*
 * zimg's depth conversion (DepthConversion, src/zimg/depth/depth.cpp:43-66) of
 * one plane: pixel formats as zimg's PixelFormat (type 0 BYTE, 1 WORD, 2
 * HALF, 3 FLOAT), dither as DitherType, `plane` the plane index (0-3) that
 * selects the dither table's variant; cpu as ref_plan_create.
 */
int ref_depth_convert(int in_type, unsigned in_depth, int in_full, int in_chroma, int out_type, unsigned out_depth,
                      int out_full, int out_chroma, int dither, unsigned plane, int cpu, unsigned w, unsigned h,
                      const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, char *err, size_t errlen)
{
	try {
		const zimg::PixelFormat fin(static_cast<PixelType>(in_type), in_depth, in_full != 0, in_chroma != 0);
		const zimg::PixelFormat fout(static_cast<PixelType>(out_type), out_depth, out_full != 0, out_chroma != 0);
		std::array<bool, 4> planes{};
		planes[plane & 3] = true;
		zimg::depth::DepthConversion conv(w, h);
		conv.set_pixel_in(fin)
			.set_pixel_out(fout)
			.set_dither_type(static_cast<zimg::depth::DitherType>(dither))
			.set_planes(planes)
			.set_cpu(make_cpu(cpu));
		zimg::depth::DepthConversion::result res = conv.create();
		const graphengine::Filter *f = res.filter_refs[plane & 3];
		if (!f) {
			const size_t bytes = static_cast<size_t>(w) * zimg::pixel_size(fout.type);
			for (unsigned i = 0; i < h; ++i)
				std::memcpy(static_cast<char *>(dst) + i * dst_stride, static_cast<const char *>(src) + i * src_stride,
				            bytes);
			return 0;
		}
		run_filter(*f, src, src_stride, dst, dst_stride);
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

/*
 * zimg's UnresizeConversion (src/zimg/unresize/unresize.h:96-114,
 * unresize.cpp:34-91) on one FLOAT plane, its filters driven over the whole
 * plane; the intermediate of two passes lives in an aligned buffer.
 */
int ref_unresize_plane(unsigned up_w, unsigned up_h, unsigned orig_w, unsigned orig_h, double shift_w, double shift_h,
                       int cpu, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, char *err,
                       size_t errlen)
{
	try {
		zimg::unresize::UnresizeConversion conv(up_w, up_h, PixelType::FLOAT);
		conv.set_orig_width(orig_w).set_orig_height(orig_h).set_shift_w(shift_w).set_shift_h(shift_h).set_cpu(make_cpu(cpu));
		auto pair = conv.create();
		if (!pair.first) {
			for (unsigned i = 0; i < up_h; ++i)
				std::memcpy(static_cast<char *>(dst) + i * dst_stride, static_cast<const char *>(src) + i * src_stride,
				            static_cast<size_t>(up_w) * 4);
			return 0;
		}
		if (!pair.second) {
			run_filter(*pair.first, src, src_stride, dst, dst_stride);
			return 0;
		}
		const graphengine::FilterDescriptor &d = pair.first->descriptor();
		ptrdiff_t tmp_stride = (static_cast<ptrdiff_t>(d.format.width) * 4 + 63) & ~static_cast<ptrdiff_t>(63);
		void *tmp = aligned_buf(static_cast<size_t>(tmp_stride) * (d.format.height + 1));
		if (!tmp)
			throw std::bad_alloc{};
		run_filter(*pair.first, src, src_stride, tmp, tmp_stride);
		run_filter(*pair.second, tmp, tmp_stride, dst, dst_stride);
		std::free(tmp);
		return 0;
	} catch (...) {
		return catch_all(err, errlen);
	}
}

} // extern "C"
