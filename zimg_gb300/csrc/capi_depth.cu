// C ABI: depth conversion objects (zg_depth_*), zimg's DepthConversion on
// device planes. The choice of conversion and its constants follow
// src/zimg/depth/depth.cpp:43-66 and quantize.h:19-45.
#include <cstdint>
#include <cstdlib>
#include <string>

#include "capi_common.h"
#include "depth.h"

using namespace zg;

struct zg_depth {
	int device = 0;
	zg_depth_params params{};
	int mode = 0;  // 0 copy, 1 left shift, 2 to float, 3 dither
	unsigned shift = 0;
	float scale = 1.0f, offset = 0.0f, vmax = 0.0f;
	// error diffusion: the plane's wavefront shape (pointers set per call)
	EdPlane ed{};
	int ed_warps = 0, ed_ring = 0;
};

namespace {

int type_code(zg_pixel_type t)
{
	switch (t) {
	case ZG_PIXEL_BYTE: return 0;
	case ZG_PIXEL_WORD: return 1;
	case ZG_PIXEL_HALF: return 2;
	case ZG_PIXEL_FLOAT: return 3;
	default: throw Error(kErrEnumOutOfRange, "unrecognized pixel type");
	}
}

unsigned type_bits(int code)
{
	return code == 0 ? 8 : (code == 3 ? 32 : 16);
}

unsigned type_bytes(int code)
{
	return code == 0 ? 1 : (code == 3 ? 4 : 2);
}

bool is_float(int code)
{
	return code == 2 || code == 3;
}

// integer_offset / integer_range (quantize.h:19-32)
double fmt_offset(const zg_pixel_format &f, int code)
{
	if (is_float(code))
		return 0.0;
	if (f.chroma)
		return static_cast<double>(1L << (f.depth - 1));
	if (!f.fullrange)
		return static_cast<double>(16L << (f.depth - 8));
	return 0.0;
}

double fmt_range(const zg_pixel_format &f, int code)
{
	if (is_float(code))
		return 1.0;
	if (f.fullrange)
		return static_cast<double>((1L << f.depth) - 1);
	if (f.chroma && !f.ycgco)
		return static_cast<double>(224L << (f.depth - 8));
	return static_cast<double>(219L << (f.depth - 8));
}

// PixelFormat equality (common/pixel.h:194-199)
bool fmt_equal(const zg_pixel_format &a, int ca, const zg_pixel_format &b, int cb)
{
	if (is_float(ca))
		return ca == cb && !a.chroma == !b.chroma;
	return ca == cb && a.depth == b.depth && !a.fullrange == !b.fullrange && !a.chroma == !b.chroma;
}

zg_pixel_format normalised(const zg_pixel_format &f, int code)
{
	zg_pixel_format g = f;
	if (!g.depth)
		g.depth = type_bits(code);
	if (g.depth > type_bits(code))
		throw Error(kErrBitDepthOverflow, "bit depth exceeds limits of type");
	return g;
}

bool aligned(const void *p, ptrdiff_t stride, unsigned a)
{
	return reinterpret_cast<uintptr_t>(p) % a == 0 && stride % a == 0;
}

} // namespace

namespace zg {

bool depth_ed_plane(const ::zg_depth *d, EdPlane *plane, int *in_type, int *out_type)
{
	if (!d || d->mode != 3 || d->params.dither_type != ZG_DITHER_ERROR_DIFFUSION)
		return false;
	*plane = d->ed;
	*in_type = type_code(d->params.pixel_in.type);
	*out_type = type_code(d->params.pixel_out.type);
	return true;
}

} // namespace zg

extern "C" {

zg_error_code zg_depth_create(const zg_depth_params *params, zg_depth **out)
{
	return guarded([&] {
		if (!params || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = nullptr;
		const zg_depth_params &q = *params;
		if (!q.width || !q.height)
			throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
		const int ci = type_code(q.pixel_in.type), co = type_code(q.pixel_out.type);
		if (q.dither_type < ZG_DITHER_NONE || q.dither_type > ZG_DITHER_ERROR_DIFFUSION)
			throw Error(kErrEnumOutOfRange, "unrecognized dither type");
		const zg_pixel_format fi = normalised(q.pixel_in, ci), fo = normalised(q.pixel_out, co);
		if ((!fi.fullrange && fi.depth < 8) || (!fo.fullrange && fo.depth < 8))
			throw Error(kErrBitDepthOverflow, "bit depth must be at least 8 for limited range");

		auto d = std::make_unique<zg_depth>();
		d->params = q;
		d->params.pixel_in = fi;
		d->params.pixel_out = fo;
		if (fmt_equal(fi, ci, fo, co)) {
			d->mode = 0;
		} else if (!is_float(ci) && !is_float(co) && !fi.fullrange && !fo.fullrange && !fi.chroma == !fo.chroma &&
		           fo.depth >= fi.depth) {
			d->mode = 1;
			d->shift = fo.depth - fi.depth;
		} else if (is_float(co)) {
			d->mode = (is_float(ci) && ci == co) ? 0 : 2;
		} else {
			d->mode = 3;
		}
		// get_scale_offset (quantize.h:34-45): FP64, rounded to float
		const double ri = fmt_range(fi, ci), oi = fmt_offset(fi, ci), ro = fmt_range(fo, co), oo = fmt_offset(fo, co);
		d->scale = static_cast<float>(ro / ri);
		d->offset = static_cast<float>(-oi * ro / ri + oo);
		d->vmax = static_cast<float>((1UL << fo.depth) - 1);
		if (d->mode == 3 && q.dither_type == ZG_DITHER_ERROR_DIFFUSION) {
			d->ed.width = static_cast<int>(q.width);
			d->ed.height = static_cast<int>(q.height);
			d->ed.scale = d->scale;
			d->ed.offset = d->offset;
			d->ed.vmax = d->vmax;
			d->ed_warps = ed_choose_warps(d->ed.width, d->ed.height);
			// tuning override: warps per block (a bad value fails below)
			if (const char *env = std::getenv("ZG_ED_WARPS"))
				d->ed_warps = std::atoi(env);
			if (q.width > (1u << 30) || q.height > (1u << 30) || !d->ed_warps ||
			    !ed_shape(d->ed, d->ed_warps, &d->ed_ring))
				throw Error(kErrUnsupported, "plane too wide for error diffusion in this library");
		}
		d->device = current_device();
		*out = d.release();
	});
}

void zg_depth_free(zg_depth *d)
{
	delete d;
}

zg_error_code zg_depth_get_info(const zg_depth *d, int *mode)
{
	return guarded([&] {
		if (!d || !mode)
			throw Error(kErrIllegalArgument, "null pointer");
		*mode = d->mode;
	});
}

zg_error_code zg_depth_process(const zg_depth *d, const void *src, ptrdiff_t src_stride, void *dst,
                               ptrdiff_t dst_stride, zg_stream stream)
{
	return guarded([&] {
		if (!d)
			throw Error(kErrIllegalArgument, "null pointer");
		if (current_device() != d->device)
			throw Error(kErrLogic, "object used on a different device than the one it was created on");
		const zg_depth_params &q = d->params;
		const int ci = type_code(q.pixel_in.type), co = type_code(q.pixel_out.type);
		const unsigned bi = type_bytes(ci), bo = type_bytes(co);
		auto check = [](const void *p, ptrdiff_t stride, unsigned w, unsigned b, const char *what) {
			if (!p)
				throw Error(kErrIllegalArgument, std::string(what) + " is null");
			if (abs_stride(stride) < static_cast<ptrdiff_t>(w) * static_cast<ptrdiff_t>(b))
				throw Error(kErrIllegalArgument, std::string(what) + " stride smaller than a line");
			if (reinterpret_cast<uintptr_t>(p) % b || stride % b)
				throw Error(kErrIllegalArgument, std::string(what) + " not aligned to the sample size");
		};
		check(src, src_stride, q.width, bi, "src");
		check(dst, dst_stride, q.width, bo, "dst");
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		if (d->mode == 0) {
			copy_plane(dst, dst_stride, src, src_stride, static_cast<size_t>(q.width) * bo, q.height, st);
			return;
		}
		if (d->mode == 3 && q.dither_type == ZG_DITHER_ERROR_DIFFUSION) {
			EdLaunch E{};
			E.planes[0] = d->ed;
			E.planes[0].src = src;
			E.planes[0].src_stride = src_stride;
			E.planes[0].dst = dst;
			E.planes[0].dst_stride = dst_stride;
			E.num_planes = 1;
			E.in_type = ci;
			E.out_type = co;
			E.warps = d->ed_warps;
			E.ring = d->ed_ring;
			cuda_check(launch_error_diffusion(E, st), "error diffusion launch");
			return;
		}
		DepthLaunch L{};
		L.src = src;
		L.src_stride = src_stride;
		L.dst = dst;
		L.dst_stride = dst_stride;
		L.width = static_cast<int>(q.width);
		L.height = static_cast<int>(q.height);
		L.scale = d->scale;
		L.offset = d->offset;
		L.vmax = d->vmax;
		L.shift = d->shift;
		L.seq = q.plane;
		L.dither = q.dither_type == ZG_DITHER_ORDERED ? 1 : (q.dither_type == ZG_DITHER_RANDOM ? 2 : 0);
		// 8 samples per vector: 8-byte loads of BYTE, 16-byte loads of WORD, HALF and FLOAT
		L.vec_in = aligned(src, src_stride, bi == 1 ? 8 : 16);
		L.vec_out = aligned(dst, dst_stride, bo == 1 ? 8 : 16);
		cuda_check(launch_depth(ci, co, d->mode, L, st), "depth conversion launch");
	});
}

} // extern "C"
