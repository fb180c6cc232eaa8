// C ABI: the resize subset of zimg's format-level graph, with the depth
// conversions the graph puts around resize.
//
// The per-plane geometry follows zimg's graph builder: chroma planes from luma
// (graphbuilder.cpp:331-346), siting and field-parity offsets
// (graphbuilder.cpp:65-188,348-366), active-region defaults (zimg.cpp:388-397),
// subrectangle copies (graphbuilder.cpp:540-573) and the shift / subwidth
// mapping of resize_plane (graphbuilder.cpp:769-776).
#include "capi_common.h"
#include "alpha.h"
#include "depth.h"
#include "colorspace_plan.h"

#include <cfloat>
#include <cmath>
#include <vector>

using namespace zg;

namespace {

enum { PLANE_Y = 0, PLANE_U = 1, PLANE_V = 2, PLANE_A = 3 };
enum { COLOR_GREY = 0, COLOR_RGB = 1, COLOR_YUV = 2 };
enum { PARITY_PROGRESSIVE = 0, PARITY_TOP = 1, PARITY_BOTTOM = 2 };

struct PlaneGeom {
	unsigned width = 0, height = 0;
	double left = 0, top = 0, aw = 0, ah = 0;

	bool operator==(const PlaneGeom &o) const
	{
		return width == o.width && height == o.height && left == o.left && top == o.top && aw == o.aw && ah == o.ah;
	}
};

struct FormatState {
	unsigned width, height;
	int pixel_type;
	unsigned depth;
	unsigned subsample_w, subsample_h;
	int color;
	int matrix, transfer, primaries;
	int range;
	int parity;
	int chroma_location;
	int alpha;
	csp::Space cs;  // matrix, transfer, primaries as zimg's internal values
	PlaneGeom planes[4];
};

const unsigned kApi20 = ZG_MAKE_API_VERSION(2, 0);
const unsigned kApi21 = ZG_MAKE_API_VERSION(2, 1);
const unsigned kApi24 = ZG_MAKE_API_VERSION(2, 4);
const unsigned kImageDimensionMax = 1U << 30;  // 64-bit hosts (graphbuilder.cpp:23-27)

unsigned pixel_depth_max(int type)
{
	switch (type) {
	case ZG_PIXEL_BYTE: return 8;
	case ZG_PIXEL_WORD: return 16;
	case ZG_PIXEL_HALF: return 16;
	case ZG_PIXEL_FLOAT: return 32;
	default: throw Error(kErrEnumOutOfRange, "unrecognized pixel type");
	}
}

// Chroma offset from a centred sample, in chroma pixels (graphbuilder.cpp:65-110).
double offset_w(bool left_sited, double subsampling)
{
	return left_sited ? -0.5 + 0.5 * subsampling : 0.0;
}

double offset_h(int loc_h, double subsampling)
{
	if (loc_h == 1)  // top
		return -0.5 + 0.5 * subsampling;
	if (loc_h == 2)  // bottom
		return 0.5 - 0.5 * subsampling;
	return 0.0;
}

// Field offsets relative to a progressive frame of field size
// (graphbuilder.cpp:112-188).
double parity_adjust(int parity, double offset)
{
	if (parity == PARITY_TOP)
		return -0.25 + offset / 2;
	if (parity == PARITY_BOTTOM)
		return 0.25 + offset / 2;
	return offset;
}

double luma_parity(int parity)
{
	return parity == PARITY_TOP ? -0.25 : (parity == PARITY_BOTTOM ? 0.25 : 0.0);
}

// zimg_chroma_location_e -> (left-sited?, vertical: 0 centre, 1 top, 2 bottom)
// (zimg.cpp:214-236).
void chroma_location(int loc, bool *left, int *vert)
{
	switch (loc) {
	case 0: *left = true; *vert = 0; return;   // LEFT (MPEG-2)
	case 1: *left = false; *vert = 0; return;  // CENTER
	case 2: *left = true; *vert = 1; return;   // TOP_LEFT
	case 3: *left = false; *vert = 1; return;  // TOP
	case 4: *left = true; *vert = 2; return;   // BOTTOM_LEFT
	case 5: *left = false; *vert = 2; return;  // BOTTOM
	default: throw Error(kErrEnumOutOfRange, "unrecognized chroma location");
	}
}

FormatState import_format(const zg_image_format &f)
{
	if (f.version < kApi20)
		throw Error(kErrIllegalArgument, "API version invalid");
	FormatState s{};
	s.width = f.width;
	s.height = f.height;
	s.pixel_type = f.pixel_type;
	s.depth = f.depth ? f.depth : pixel_depth_max(f.pixel_type);
	s.subsample_w = f.subsample_w;
	s.subsample_h = f.subsample_h;
	s.color = f.color_family;
	if (s.color < COLOR_GREY || s.color > COLOR_YUV)
		throw Error(kErrEnumOutOfRange, "unrecognized color family");
	s.matrix = f.matrix_coefficients;
	s.transfer = f.transfer_characteristics;
	s.primaries = f.color_primaries;
	s.range = f.pixel_range;
	if (s.range != 0 && s.range != 1)
		throw Error(kErrEnumOutOfRange, "unrecognized pixel range");
	s.parity = f.field_parity;
	if (s.parity < PARITY_PROGRESSIVE || s.parity > PARITY_BOTTOM)
		throw Error(kErrEnumOutOfRange, "unrecognized field parity");
	s.chroma_location = f.chroma_location;
	s.alpha = f.version >= kApi24 ? f.alpha : 0;
	if (s.alpha < 0 || s.alpha > 2)
		throw Error(kErrEnumOutOfRange, "unrecognized alpha type");
	// translate_matrix / _transfer / _primaries (zimg.cpp:238-305,425-431)
	s.cs = csp::from_api(s.matrix, s.transfer, s.primaries);
	// colour family against matrix (validate_state, graphbuilder.cpp:199-216)
	if (s.color == COLOR_GREY && s.cs.m == csp::M_RGB)
		throw Error(kErrColorFamilyMismatch, "GREY color family cannot have RGB matrix coefficients");
	if (s.color == COLOR_RGB && s.cs.m != csp::M_UNSPEC && s.cs.m != csp::M_RGB)
		throw Error(kErrColorFamilyMismatch, "RGB color family cannot have YUV matrix coefficients");
	if (s.color == COLOR_YUV && s.cs.m == csp::M_RGB)
		throw Error(kErrColorFamilyMismatch, "YUV color family cannot have RGB matrix coefficients");

	double al = 0.0, at = 0.0, aw = s.width, ah = s.height;
	if (f.version >= kApi21) {
		al = std::isnan(f.active_region.left) ? 0.0 : f.active_region.left;
		at = std::isnan(f.active_region.top) ? 0.0 : f.active_region.top;
		aw = std::isnan(f.active_region.width) ? static_cast<double>(s.width) : f.active_region.width;
		ah = std::isnan(f.active_region.height) ? static_cast<double>(s.height) : f.active_region.height;
	}

	// validate_state (graphbuilder.cpp:190-235)
	if (!s.width || !s.height)
		throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
	if (s.width > kImageDimensionMax || s.height > kImageDimensionMax)
		throw Error(kErrInvalidImageSize, "image dimensions exceed implementation limit");
	if (s.color == COLOR_GREY && (s.subsample_w || s.subsample_h))
		throw Error(kErrGreyscaleSubsampling, "cannot subsample greyscale image");
	if (s.color == COLOR_RGB && (s.subsample_w || s.subsample_h))
		throw Error(kErrUnsupportedSubsampling, "subsampled RGB image not supported");
	if (s.subsample_h > 1 && s.parity != PARITY_PROGRESSIVE)
		throw Error(kErrUnsupportedSubsampling, "interlaced vertical subsampling greater than 2x is not supported");
	if (s.subsample_w > 2 || s.subsample_h > 2)
		throw Error(kErrUnsupportedSubsampling, "subsampling greater than 4x is not supported");
	if (s.width % (1u << s.subsample_w) || s.height % (1u << s.subsample_h))
		throw Error(kErrImageNotDivisible, "image dimensions must be divisible by subsampling factor");
	if (s.depth > pixel_depth_max(s.pixel_type))
		throw Error(kErrBitDepthOverflow, "bit depth exceeds limits of type");
	if (s.pixel_type != ZG_PIXEL_FLOAT && s.pixel_type != ZG_PIXEL_HALF && s.range == 0 && s.depth < 8)
		throw Error(kErrBitDepthOverflow, "bit depth must be at least 8 for limited range");
	if (!std::isfinite(al) || !std::isfinite(at) || !std::isfinite(aw) || !std::isfinite(ah))
		throw Error(kErrInvalidImageSize, "active window must be finite");
	if (aw <= 0 || ah <= 0)
		throw Error(kErrInvalidImageSize, "active window must be positive");

	// Planes (graphbuilder.cpp:331-366).
	PlaneGeom y{ s.width, s.height, al, at, aw, ah };
	s.planes[PLANE_Y] = y;
	if (s.color != COLOR_GREY) {
		const double sw = 1.0 / (1UL << s.subsample_w);
		const double sh = 1.0 / (1UL << s.subsample_h);
		PlaneGeom u{ s.width >> s.subsample_w, s.height >> s.subsample_h, al * sw, at * sh, aw * sw, ah * sh };
		s.planes[PLANE_U] = u;
		s.planes[PLANE_V] = u;
	}
	if (s.alpha)
		s.planes[PLANE_A] = s.planes[PLANE_Y];

	s.planes[PLANE_Y].top -= luma_parity(s.parity);
	if (s.color != COLOR_GREY) {
		bool left_sited = false;
		int vert = 0;
		chroma_location(s.chroma_location, &left_sited, &vert);
		const double subscale_w = static_cast<double>(s.planes[PLANE_U].width) / s.planes[PLANE_Y].width;
		const double subscale_h = static_cast<double>(s.planes[PLANE_U].height) / s.planes[PLANE_Y].height;
		const double ow = offset_w(left_sited, subscale_w);
		const double oh = parity_adjust(s.parity, offset_h(vert, subscale_h));
		for (int p : { PLANE_U, PLANE_V }) {
			s.planes[p].left -= ow;
			s.planes[p].top -= oh;
		}
	}
	if (s.alpha)
		s.planes[PLANE_A].top -= luma_parity(s.parity);
	return s;
}

} // namespace

namespace {

// A plane's pixel format (zimg's PixelFormat, common/pixel.h:135-181).
struct PixFmt {
	int type;
	unsigned depth;
	bool full, chroma;
};

bool fmt_equal(const PixFmt &a, const PixFmt &b)
{
	// common/pixel.h:194-199: floats compare by type and chroma only
	if (a.type == ZG_PIXEL_FLOAT || a.type == ZG_PIXEL_HALF)
		return a.type == b.type && a.chroma == b.chroma;
	return a.type == b.type && a.depth == b.depth && a.full == b.full && a.chroma == b.chroma;
}

// The format resize runs in (choose_resize_format, graphbuilder.cpp:720-751),
// resize supporting WORD and FLOAT.
PixFmt choose_resize_format(const PixFmt &s, const PixFmt &d, double src_pels, double dst_pels)
{
	auto supported = [](int t) { return t == ZG_PIXEL_WORD || t == ZG_PIXEL_FLOAT; };
	if (supported(s.type) && supported(d.type))
		return src_pels < dst_pels ? d : s;
	if (supported(s.type))
		return s;
	if (supported(d.type))
		return d;
	if (s.type == ZG_PIXEL_BYTE && !s.full)
		return PixFmt{ ZG_PIXEL_WORD, 16, false, s.chroma };
	return PixFmt{ ZG_PIXEL_FLOAT, 32, false, false };
}

size_t pitch_of(unsigned w, unsigned bytes)
{
	return (static_cast<size_t>(w) * bytes + 255) & ~static_cast<size_t>(255);
}

zg_depth *make_depth(unsigned w, unsigned h, const PixFmt &in, const PixFmt &out, int dither, int plane)
{
	zg_depth_params q{};
	q.width = w;
	q.height = h;
	q.pixel_in = zg_pixel_format{ static_cast<zg_pixel_type>(in.type), in.depth, in.full, in.chroma, 0 };
	q.pixel_out = zg_pixel_format{ static_cast<zg_pixel_type>(out.type), out.depth, out.full, out.chroma, 0 };
	q.dither_type = static_cast<zg_dither_type>(dither);
	q.plane = static_cast<unsigned>(plane);
	zg_depth *d = nullptr;
	zg_error_code rc = zg_depth_create(&q, &d);
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[256];
		zg_get_last_error(msg, sizeof(msg));
		throw Error(rc, msg);
	}
	return d;
}

// The resize of one plane between two geometries (resize_plane,
// graphbuilder.cpp:769-776).
zg_resize_params geom_resize_params(const PlaneGeom &sp, const PlaneGeom &dp)
{
	zg_resize_params rp;
	zg_resize_params_default(&rp);
	const double scale_w = dp.aw / sp.aw;
	const double scale_h = dp.ah / sp.ah;
	rp.src_width = sp.width;
	rp.src_height = sp.height;
	rp.dst_width = dp.width;
	rp.dst_height = dp.height;
	rp.shift_w = sp.left - dp.left / scale_w;
	rp.shift_h = sp.top - dp.top / scale_h;
	rp.subwidth = sp.aw * (dp.width / dp.aw);
	rp.subheight = sp.ah * (dp.height / dp.ah);
	return rp;
}

zg_resize *make_float_resize(const PlaneGeom &sp, const PlaneGeom &dp, int filter, double a, double b, size_t *tmp)
{
	zg_resize_params rp = geom_resize_params(sp, dp);
	rp.pixel_type = ZG_PIXEL_FLOAT;
	rp.depth = 32;
	rp.filter = static_cast<zg_resample_filter>(filter);
	rp.filter_param_a = a;
	rp.filter_param_b = b;
	zg_resize *r = nullptr;
	zg_error_code rc = zg_resize_create(&rp, &r);
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[256];
		zg_get_last_error(msg, sizeof(msg));
		throw Error(rc, msg);
	}
	size_t t = 0;
	zg_resize_get_tmp_size(r, &t);
	*tmp = std::max(*tmp, t);
	return r;
}

void run_resize(const zg_resize *r, const void *src, ptrdiff_t ss, void *dst, ptrdiff_t ds, void *tmp, zg_stream st)
{
	zg_error_code rc = zg_resize_process(r, src, ss, dst, ds, tmp, st);
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[256];
		zg_get_last_error(msg, sizeof(msg));
		throw Error(rc, msg);
	}
}

// needs_interpolation_plane (graphbuilder.cpp:509-525): another active size
// or another fractional phase of the active region's corner
bool needs_interpolation_plane(const PlaneGeom &a, const PlaneGeom &b)
{
	auto phase = [](double x) {
		double ip;
		return std::modf(x, &ip);
	};
	return a.aw != b.aw || a.ah != b.ah || phase(a.left) != phase(b.left) || phase(a.top) != phase(b.top);
}

void run_depth(const zg_depth *d, const void *src, ptrdiff_t ss, void *dst, ptrdiff_t ds, zg_stream st)
{
	zg_error_code rc = zg_depth_process(d, src, ss, dst, ds, st);
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[256];
		zg_get_last_error(msg, sizeof(msg));
		throw Error(rc, msg);
	}
}

// One plane from one geometry and pixel format to another, as zimg's
// connect_plane does it (graphbuilder.cpp:892-953): a depth conversion into
// the format resize works in (choose_resize_format), the resize, a depth
// conversion to the output format; a copy or a depth conversion alone when
// the geometry is kept. Its scratch (the intermediate planes and the
// resize's tmp) is `scratch` bytes.
struct Chain {
	int kind = 0;  // 0 copy, 1 depth only, 2 resize
	unsigned sw = 0, sh = 0, dw = 0, dh = 0, in_bytes = 0, out_bytes = 0;
	zg_depth *pre = nullptr, *post = nullptr, *only = nullptr;
	zg_resize *resize = nullptr;
	size_t pre_pitch = 0, mid_pitch = 0, off_mid = 0, off_rtmp = 0, scratch = 0;

	void release()
	{
		zg_depth_free(pre);
		zg_depth_free(post);
		zg_depth_free(only);
		zg_resize_free(resize);
		pre = post = only = nullptr;
		resize = nullptr;
	}
};

unsigned sample_bytes(int t)
{
	return t == ZG_PIXEL_BYTE ? 1u : (t == ZG_PIXEL_FLOAT ? 4u : 2u);
}

Chain make_chain(const PlaneGeom &sp, const PlaneGeom &dp, const PixFmt &fs, const PixFmt &fd, int filter, double a,
                 double b, int dither, int plane)
{
	Chain c;
	c.sw = sp.width;
	c.sh = sp.height;
	c.dw = dp.width;
	c.dh = dp.height;
	c.in_bytes = sample_bytes(fs.type);
	c.out_bytes = sample_bytes(fd.type);
	if (sp == dp) {
		if (!fmt_equal(fs, fd)) {
			c.kind = 1;
			c.only = make_depth(dp.width, dp.height, fs, fd, dither, plane);
		}
		return c;
	}
	c.kind = 2;
	const PixFmt fr = choose_resize_format(fs, fd, static_cast<double>(sp.width) * sp.height,
	                                       static_cast<double>(dp.width) * dp.height);
	zg_resize_params rp = geom_resize_params(sp, dp);
	rp.pixel_type = static_cast<zg_pixel_type>(fr.type);
	rp.depth = fr.type == ZG_PIXEL_FLOAT ? 32 : fr.depth;
	rp.filter = static_cast<zg_resample_filter>(filter);
	rp.filter_param_a = a;
	rp.filter_param_b = b;
	zg_error_code rc = zg_resize_create(&rp, &c.resize);
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[256];
		zg_get_last_error(msg, sizeof(msg));
		throw Error(rc, msg);
	}
	size_t rtmp = 0;
	zg_resize_get_tmp_size(c.resize, &rtmp);
	size_t off = 0;
	if (!fmt_equal(fs, fr)) {
		c.pre = make_depth(sp.width, sp.height, fs, fr, dither, plane);
		c.pre_pitch = pitch_of(sp.width, sample_bytes(fr.type));
		off += c.pre_pitch * sp.height;
	}
	if (!fmt_equal(fr, fd)) {
		c.post = make_depth(dp.width, dp.height, fr, fd, dither, plane);
		c.mid_pitch = pitch_of(dp.width, sample_bytes(fr.type));
		c.off_mid = off;
		off += c.mid_pitch * dp.height;
	}
	c.off_rtmp = off;
	c.scratch = off + rtmp;
	return c;
}

void run_chain(const Chain &c, const void *src, ptrdiff_t ss, void *dst, ptrdiff_t ds, char *scratch, zg_stream st)
{
	if (c.kind == 0) {
		copy_plane(dst, ds, src, ss, static_cast<size_t>(c.dw) * c.out_bytes, c.dh, reinterpret_cast<cudaStream_t>(st));
		return;
	}
	if (c.kind == 1) {
		run_depth(c.only, src, ss, dst, ds, st);
		return;
	}
	const void *rs = src;
	ptrdiff_t rss = ss;
	if (c.pre) {
		run_depth(c.pre, src, ss, scratch, static_cast<ptrdiff_t>(c.pre_pitch), st);
		rs = scratch;
		rss = static_cast<ptrdiff_t>(c.pre_pitch);
	}
	void *rd = c.post ? static_cast<void *>(scratch + c.off_mid) : dst;
	const ptrdiff_t rds = c.post ? static_cast<ptrdiff_t>(c.mid_pitch) : ds;
	run_resize(c.resize, rs, rss, rd, rds, scratch + c.off_rtmp, st);
	if (c.post)
		run_depth(c.post, rd, rds, dst, ds, st);
}

// Error-diffusion conversions of a frame's planes, side by side: one launch
// per run of up to kEdMaxPlanes planes of the same pixel types, every block
// with the most warps any of them wants; a plane whose shape does not fit
// that launch runs on its own.
template <class D>
void run_ed_planes(const D *items, int n, zg_stream stream)
{
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	std::vector<bool> done(n, false);
	for (int a = 0; a < n; ++a) {
		if (done[a])
			continue;
		EdPlane pa;
		int it = 0, ot = 0;
		depth_ed_plane(items[a].d, &pa, &it, &ot);
		std::vector<int> group{ a };
		for (int b = a + 1; b < n && static_cast<int>(group.size()) < kEdMaxPlanes; ++b) {
			EdPlane pb;
			int it2 = 0, ot2 = 0;
			if (!done[b] && depth_ed_plane(items[b].d, &pb, &it2, &ot2) && it2 == it && ot2 == ot)
				group.push_back(b);
		}
		int warps = 1;
		for (int k : group) {
			EdPlane q;
			int i2 = 0, o2 = 0;
			depth_ed_plane(items[k].d, &q, &i2, &o2);
			warps = std::max(warps, ed_choose_warps(q.width, q.height));
		}
		EdLaunch E{};
		E.in_type = it;
		E.out_type = ot;
		E.warps = warps;
		E.ring = 1;
		bool ok = true;
		for (int k : group) {
			EdPlane q;
			int i2 = 0, o2 = 0;
			depth_ed_plane(items[k].d, &q, &i2, &o2);
			int ring = 0;
			ok = ok && ed_shape(q, warps, &ring);
			q.src = items[k].src;
			q.src_stride = items[k].ss;
			q.dst = items[k].dst;
			q.dst_stride = items[k].ds;
			E.planes[E.num_planes++] = q;
			E.ring = std::max(E.ring, ring);
		}
		ok = ok && ed_smem_bytes(warps, E.ring) <= 227 * 1024;
		if (ok) {
			cuda_check(launch_error_diffusion(E, st), "error diffusion launch");
		} else {
			for (int k : group)
				run_depth(items[k].d, items[k].src, items[k].ss, items[k].dst, items[k].ds, stream);
		}
		for (int k : group)
			done[k] = true;
	}
}

// needs_colorspace (graphbuilder.cpp:484-506)
bool needs_colorspace(const FormatState &s, const FormatState &d)
{
	if (s.cs == d.cs)
		return false;
	if (s.cs.t == d.cs.t && s.cs.p == d.cs.p) {
		if (s.color == COLOR_GREY)
			return false;  // GREY to YUV / RGB: value-initialised or duplicated planes
		if (s.color != COLOR_RGB && d.color == COLOR_GREY)
			return false;  // YUV / GREY to GREY: chroma dropped
	}
	return true;
}

} // namespace

struct zg_graph {
	int device;
	struct Plane {
		bool present = false;      // read, written or both
		bool has_src = false, has_dst = false;
		int mode = 0;  // 0 copy, 1 copy subrectangle, 2 resize, 3 depth only, 4 depth of a subrectangle,
		               // 5 straight-alpha chain, 6 colorspace chain, 7 made from other planes
		unsigned w = 0, h = 0;      // output size
		unsigned off_x = 0, off_y = 0;
		unsigned in_bytes = 0, out_bytes = 0;
		zg_resize_params params{};
		zg_resize *resize = nullptr;
		zg_unresize *unresize = nullptr;  // instead of resize when the filter is ZG_RESIZE_UNRESIZE
		// depth conversions around resize (graphbuilder.cpp:943-950): into
		// the resize format before, to the output format after; their
		// planes live in tmp (pre at 0, mid next, resize scratch last)
		zg_depth *pre = nullptr, *post = nullptr, *only = nullptr;
		size_t pre_pitch = 0, mid_pitch = 0, off_mid = 0, off_tmp = 0;
		// the last step diffuses errors: it runs after every plane's other
		// steps, in one launch with the frame's other such planes (a resize
		// before it writes into a region of tmp of the plane's own)
		bool ed_last = false;
		size_t off_mid_own = 0;
		size_t tmp = 0;
		// ring-buffer (line-masked) planes: the plane's full size, its
		// vertical subsampling shift, and whole-plane staging copies in tmp
		unsigned src_w = 0, src_h = 0, src_ssh = 0, dst_ssh = 0;
		size_t sstage_pitch = 0, dstage_pitch = 0, off_sstage = 0, off_dstage = 0;
	} planes[4];
	// Straight alpha through an interpolating resize (connect_internal,
	// graphbuilder.cpp:1019-1068): every plane to FLOAT 4:4:4 at the source
	// luma geometry (chroma resized up), colour planes multiplied by alpha,
	// all four resized to the destination luma geometry, colour divided by
	// alpha, chroma resized to its own geometry, every plane converted to the
	// output format. Float planes in tmp: four at the source luma size (slot
	// 3 alpha), four at the destination luma size when that differs, one
	// chroma plane at each end, then the resizes' scratch.
	struct Premul {
		bool on = false;
		int ncolor = 0;
		bool across_needed = false;  // source and destination luma geometry differ
		unsigned sw = 0, sh = 0, dw = 0, dh = 0;
		size_t s_pitch = 0, d_pitch = 0, off_s = 0, off_d = 0;
		zg_depth *in[4] = {}, *out[4] = {};
		zg_resize *up = nullptr;         // YUV chroma: source chroma -> source luma geometry
		zg_resize *across = nullptr;     // source -> destination luma geometry, luma filter
		zg_resize *across_uv = nullptr;  // the same with the chroma filter (YUV)
		zg_resize *down = nullptr;       // YUV chroma: destination luma -> destination chroma geometry
		unsigned cs_w = 0, cs_h = 0, cd_w = 0, cd_h = 0;
		size_t cs_pitch = 0, cd_pitch = 0, off_cs = 0, off_cd = 0, off_rtmp = 0;
	} premul;
	// A colorspace change (connect_color_channels, graphbuilder.cpp:975-1014):
	// the colour planes to FLOAT 4:4:4 at the work geometry (each dimension
	// the smaller side's), GREY duplicated into three planes, the colorspace
	// operations in place, then each output plane from the work planes to
	// its geometry and format. Work planes and the chains' shared scratch in
	// tmp from off_work.
	struct Color {
		bool on = false;
		int n_in = 0, n_out = 0;  // colour planes read / written
		unsigned ww = 0, wh = 0;
		size_t w_pitch = 0, off_work = 0, off_scratch = 0;
		Chain in[3], out[3];
		csp::Plan plan;
	} color;
	// output planes made without a source plane of their own (grey_to_yuv /
	// grey_to_rgb, graphbuilder.cpp:615-659): 1 filled with fill_value, 2 a
	// copy of the luma output
	int out_fill[4] = {};
	uint32_t fill_value = 0;
	size_t tmp_size = 0;
	// lines and widths the callbacks are called with (the luma plane's), and
	// the vertical subsampling step of the source and destination formats
	unsigned src_lines = 0, dst_lines = 0, src_width = 0, dst_width = 0, src_step = 1, dst_step = 1;

	~zg_graph()
	{
		for (auto &p : planes) {
			zg_resize_free(p.resize);
			zg_unresize_free(p.unresize);
			zg_depth_free(p.pre);
			zg_depth_free(p.post);
			zg_depth_free(p.only);
		}
		for (int p = 0; p < 4; ++p) {
			zg_depth_free(premul.in[p]);
			zg_depth_free(premul.out[p]);
		}
		zg_resize_free(premul.up);
		zg_resize_free(premul.across);
		zg_resize_free(premul.across_uv);
		zg_resize_free(premul.down);
		for (int p = 0; p < 3; ++p) {
			color.in[p].release();
			color.out[p].release();
		}
	}
};

extern "C" {

void zg_image_format_default(zg_image_format *ptr, unsigned version)
{
	// zimg_image_format_default (zimg.cpp:595-630)
	if (!ptr)
		return;
	std::memset(ptr, 0, sizeof(*ptr));
	ptr->version = version;
	ptr->pixel_type = -1;
	ptr->color_family = COLOR_GREY;
	ptr->matrix_coefficients = 2;
	ptr->transfer_characteristics = 2;
	ptr->color_primaries = 2;
	ptr->pixel_range = 0;
	ptr->field_parity = PARITY_PROGRESSIVE;
	ptr->chroma_location = 0;
	ptr->active_region.left = NAN;
	ptr->active_region.top = NAN;
	ptr->active_region.width = NAN;
	ptr->active_region.height = NAN;
	ptr->alpha = 0;
}

void zg_graph_builder_params_default(zg_graph_builder_params *ptr, unsigned version)
{
	// zimg_graph_builder_params_default (zimg.cpp:632-660)
	if (!ptr)
		return;
	std::memset(ptr, 0, sizeof(*ptr));
	ptr->version = version;
	ptr->resample_filter = ZG_RESIZE_BICUBIC;
	ptr->filter_param_a = NAN;
	ptr->filter_param_b = NAN;
	ptr->resample_filter_uv = ZG_RESIZE_BILINEAR;
	ptr->filter_param_a_uv = NAN;
	ptr->filter_param_b_uv = NAN;
	ptr->dither_type = 0;
	ptr->cpu_type = 1;
	ptr->nominal_peak_luminance = NAN;
}

zg_graph *zg_graph_build(const zg_image_format *src_format, const zg_image_format *dst_format,
                         const zg_graph_builder_params *params)
{
	zg_graph *result = nullptr;
	guarded([&] {
		if (!src_format || !dst_format)
			throw Error(kErrIllegalArgument, "null pointer");
		if (src_format->version != dst_format->version)
			throw Error(kErrIllegalArgument, "image format versions do not match");
		FormatState s = import_format(*src_format);
		FormatState d = import_format(*dst_format);

		zg_graph_builder_params defaults;
		zg_graph_builder_params_default(&defaults, src_format->version);
		const zg_graph_builder_params &gp = params ? *params : defaults;

		const bool format_change =
			s.pixel_type != d.pixel_type || s.depth != d.depth || (s.pixel_type != ZG_PIXEL_FLOAT && s.range != d.range);
		const bool colorspace = needs_colorspace(s, d);
		if (!colorspace && s.color != d.color && !(s.color == COLOR_GREY || d.color == COLOR_GREY))
			throw Error(kErrNoColorspaceConversion, "colour family change without a colorspace conversion");
		if (colorspace && s.alpha == 1)
			throw Error(kErrUnsupported, "colorspace conversion of images with straight alpha is not supported by this library");
		if (colorspace && gp.resample_filter == ZG_RESIZE_UNRESIZE)
			throw Error(kErrUnsupported, "colorspace conversion with unresize is not supported by this library");
		if (s.alpha != d.alpha)
			throw Error(kErrUnsupported, "alpha conversion is outside the resize path");
		(void)format_change;

		auto g = std::make_unique<zg_graph>();
		g->device = current_device();
		auto bytes = [](int t) { return t == ZG_PIXEL_BYTE ? 1u : (t == ZG_PIXEL_FLOAT ? 4u : 2u); };
		const int dither = static_cast<int>(gp.dither_type);
		// A plane's pixel format: chroma of YUV centred; alpha full range in
		// the integer types, never chroma (alpha_from_luma,
		// graphbuilder.cpp:404-408)
		auto plane_fmt = [](const FormatState &f, int p) {
			if (p == PLANE_A) {
				const bool is_int = f.pixel_type == ZG_PIXEL_BYTE || f.pixel_type == ZG_PIXEL_WORD;
				return PixFmt{ f.pixel_type, f.depth, is_int, false };
			}
			const bool uv = (p == PLANE_U || p == PLANE_V) && f.color == COLOR_YUV;
			return PixFmt{ f.pixel_type, f.depth, f.range == 1, uv };
		};
		// needs_interpolation over the planes both formats have
		// (graphbuilder.cpp:527-538)
		bool interpolate = needs_interpolation_plane(s.planes[PLANE_Y], d.planes[PLANE_Y]);
		if (s.color != COLOR_GREY && d.color != COLOR_GREY)
			interpolate = interpolate || needs_interpolation_plane(s.planes[PLANE_U], d.planes[PLANE_U]) ||
			              needs_interpolation_plane(s.planes[PLANE_V], d.planes[PLANE_V]);
		if (s.alpha)
			interpolate = interpolate || needs_interpolation_plane(s.planes[PLANE_A], d.planes[PLANE_A]);
		// straight alpha is premultiplied around an interpolating resize
		// (needs_premul, graphbuilder.cpp:594-600)
		const bool premul = s.alpha == 1 && interpolate;
		if (premul && gp.resample_filter == ZG_RESIZE_UNRESIZE)
			throw Error(kErrUnsupported, "unresize of images with straight alpha is not supported by this library");

		for (int p = 0; p < 4 && premul; ++p) {
			const bool chroma = p == PLANE_U || p == PLANE_V;
			if (chroma && s.color == COLOR_GREY)
				continue;
			auto &pm = g->premul;
			const PlaneGeom &gs = s.planes[PLANE_Y], &gd = d.planes[PLANE_Y];
			if (!pm.on) {
				pm.on = true;
				pm.ncolor = s.color == COLOR_GREY ? 1 : 3;
				pm.sw = gs.width;
				pm.sh = gs.height;
				pm.dw = gd.width;
				pm.dh = gd.height;
				pm.s_pitch = pitch_of(gs.width, 4);
				pm.d_pitch = pitch_of(gd.width, 4);
				pm.across_needed = !(gs == gd);
			}
			auto &gpl = g->planes[p];
			gpl.present = gpl.has_src = gpl.has_dst = true;
			gpl.mode = 5;
			const int q = (s.color == COLOR_RGB && chroma) ? PLANE_Y : p;
			const PlaneGeom &sp = s.planes[q], &dp = d.planes[q];
			gpl.w = dp.width;
			gpl.h = dp.height;
			gpl.in_bytes = bytes(s.pixel_type);
			gpl.out_bytes = bytes(d.pixel_type);
			gpl.src_w = sp.width;
			gpl.src_h = sp.height;
			gpl.src_ssh = chroma && s.color == COLOR_YUV ? s.subsample_h : 0;
			gpl.dst_ssh = chroma && s.color == COLOR_YUV ? d.subsample_h : 0;
			const bool uv = chroma && s.color == COLOR_YUV;
			// make_float_444_state (graphbuilder.cpp:446-457)
			const PixFmt fl{ ZG_PIXEL_FLOAT, 32, false, uv };
			pm.in[p] = make_depth(sp.width, sp.height, plane_fmt(s, p), fl, dither, p);
			pm.out[p] = make_depth(dp.width, dp.height, fl, plane_fmt(d, p), dither, p);
			if (uv && !(sp == gs) && !pm.up) {
				pm.up = make_float_resize(sp, gs, gp.resample_filter_uv, gp.filter_param_a_uv, gp.filter_param_b_uv,
				                          &pm.off_rtmp);
				pm.cs_w = sp.width;
				pm.cs_h = sp.height;
			}
			if (uv && !(dp == gd) && !pm.down) {
				pm.down = make_float_resize(gd, dp, gp.resample_filter_uv, gp.filter_param_a_uv, gp.filter_param_b_uv,
				                            &pm.off_rtmp);
				pm.cd_w = dp.width;
				pm.cd_h = dp.height;
			}
			if (pm.across_needed && !pm.across)
				pm.across = make_float_resize(gs, gd, gp.resample_filter, gp.filter_param_a, gp.filter_param_b,
				                              &pm.off_rtmp);
			if (pm.across_needed && uv && !pm.across_uv)
				pm.across_uv = make_float_resize(gs, gd, gp.resample_filter_uv, gp.filter_param_a_uv,
				                                 gp.filter_param_b_uv, &pm.off_rtmp);
		}
		if (premul) {
			// tmp layout; off_rtmp held the largest resize scratch until now
			auto &pm = g->premul;
			const size_t rscratch = pm.off_rtmp;
			size_t off = 0;
			pm.off_s = off;
			off += 4 * pm.s_pitch * pm.sh;
			pm.off_d = off;
			if (pm.across_needed)
				off += 4 * pm.d_pitch * pm.dh;
			pm.cs_pitch = pitch_of(pm.cs_w, 4);
			pm.off_cs = off;
			off += pm.cs_pitch * pm.cs_h;
			pm.cd_pitch = pitch_of(pm.cd_w, 4);
			pm.off_cd = off;
			off += pm.cd_pitch * pm.cd_h;
			pm.off_rtmp = off;
			g->tmp_size = off + rscratch;
		}

		for (int p = 0; p < 4 && !premul; ++p) {
			const bool chroma = p == PLANE_U || p == PLANE_V;
			if (chroma && (s.color == COLOR_GREY || d.color == COLOR_GREY))
				continue;
			if (p == PLANE_A && !s.alpha)
				continue;
			if (colorspace && p != PLANE_A)
				continue;
			auto &gpl = g->planes[p];
			gpl.present = gpl.has_src = gpl.has_dst = true;
			// RGB planes share the luma plane's conversion (graphbuilder.cpp:892-905).
			const int q = (s.color == COLOR_RGB && chroma) ? PLANE_Y : p;
			const PlaneGeom &sp = s.planes[q];
			const PlaneGeom &dp = d.planes[q];
			gpl.w = dp.width;
			gpl.h = dp.height;
			gpl.in_bytes = bytes(s.pixel_type);
			gpl.out_bytes = bytes(d.pixel_type);
			gpl.src_w = sp.width;
			gpl.src_h = sp.height;
			gpl.src_ssh = chroma && s.color == COLOR_YUV ? s.subsample_h : 0;
			gpl.dst_ssh = chroma && s.color == COLOR_YUV ? d.subsample_h : 0;
			// plane formats; full-range BYTE kept at its depth is treated as
			// limited range for the whole chain (graphbuilder.cpp:912-920)
			PixFmt fs = plane_fmt(s, p), fd = plane_fmt(d, p);
			if (fs.type == ZG_PIXEL_BYTE && fs.full && fd.full && fs.depth == fd.depth)
				fs.full = fd.full = false;

			if (sp == dp) {
				if (fmt_equal(fs, fd)) {
					gpl.mode = 0;
				} else {
					gpl.mode = 3;
					gpl.only = make_depth(dp.width, dp.height, fs, fd, dither, p);
				}
				continue;
			}
			// Pixel-aligned subrectangle equal to the output: plain copy
			// (can_copy_tile, graphbuilder.cpp:540-573).
			{
				auto is_int = [](double x) { return std::trunc(x) == x; };
				bool tile = !(sp.aw == sp.width || sp.ah == sp.height) &&
				            dp.aw == dp.width && dp.ah == dp.height &&
				            sp.aw == dp.width && sp.ah == dp.height;
				double sl = sp.left - dp.left, st = sp.top - dp.top;
				tile = tile && is_int(sl) && is_int(st) && sl >= 0 && st >= 0 &&
				       sl + sp.aw <= sp.width && st + sp.ah <= sp.height;
				if (tile) {
					gpl.mode = fmt_equal(fs, fd) ? 1 : 4;
					gpl.off_x = static_cast<unsigned>(sl);
					gpl.off_y = static_cast<unsigned>(st);
					if (gpl.mode == 4)
						gpl.only = make_depth(dp.width, dp.height, fs, fd, dither, p);
					continue;
				}
			}
			gpl.mode = 2;
			const bool unresize = gp.resample_filter == ZG_RESIZE_UNRESIZE;
			if (unresize && (sp.aw != sp.width || sp.ah != sp.height || dp.aw != dp.width || dp.ah != dp.height))
				throw Error(kErrResamplingNotAvailable, "unresize not supported for given subregion");
			// unresize works in FLOAT (choose_resize_format, graphbuilder.cpp:722-723)
			const PixFmt fr = unresize ? PixFmt{ ZG_PIXEL_FLOAT, 32, false, false }
			                           : choose_resize_format(fs, fd, static_cast<double>(sp.width) * sp.height,
			                                                  static_cast<double>(dp.width) * dp.height);
			zg_resize_params rp = geom_resize_params(sp, dp);
			rp.pixel_type = static_cast<zg_pixel_type>(fr.type);
			rp.depth = fr.type == ZG_PIXEL_FLOAT ? 32 : fr.depth;
			rp.filter = static_cast<zg_resample_filter>(chroma && s.color == COLOR_YUV ? gp.resample_filter_uv : gp.resample_filter);
			rp.filter_param_a = chroma && s.color == COLOR_YUV ? gp.filter_param_a_uv : gp.filter_param_a;
			rp.filter_param_b = chroma && s.color == COLOR_YUV ? gp.filter_param_b_uv : gp.filter_param_b;
			gpl.params = rp;
			size_t rtmp = 0;
			zg_error_code rc;
			if (unresize) {
				const zg_unresize_params up{ sp.width, sp.height, dp.width, dp.height, rp.shift_w, rp.shift_h };
				rc = zg_unresize_create(&up, &gpl.unresize);
				if (rc == ZG_ERROR_SUCCESS)
					zg_unresize_get_tmp_size(gpl.unresize, &rtmp);
			} else {
				rc = zg_resize_create(&rp, &gpl.resize);
				if (rc == ZG_ERROR_SUCCESS)
					zg_resize_get_tmp_size(gpl.resize, &rtmp);
			}
			if (rc != ZG_ERROR_SUCCESS) {
				char msg[256];
				zg_get_last_error(msg, sizeof(msg));
				throw Error(rc, msg);
			}
			size_t off = 0;
			if (!fmt_equal(fs, fr)) {
				gpl.pre = make_depth(sp.width, sp.height, fs, fr, dither, p);
				gpl.pre_pitch = pitch_of(sp.width, bytes(fr.type));
				off += gpl.pre_pitch * sp.height;
			}
			if (!fmt_equal(fr, fd)) {
				gpl.post = make_depth(dp.width, dp.height, fr, fd, dither, p);
				gpl.mid_pitch = pitch_of(dp.width, bytes(fr.type));
				gpl.off_mid = off;
				off += gpl.mid_pitch * dp.height;
			}
			gpl.off_tmp = off;
			gpl.tmp = off + rtmp;
			g->tmp_size = std::max(g->tmp_size, gpl.tmp);
		}
		{
			size_t off = (g->tmp_size + 255) & ~static_cast<size_t>(255);
			for (auto &gpl : g->planes) {
				EdPlane ep;
				int it = 0, ot = 0;
				if ((gpl.mode == 3 || gpl.mode == 4) && depth_ed_plane(gpl.only, &ep, &it, &ot)) {
					gpl.ed_last = true;
				} else if (gpl.mode == 2 && gpl.post && depth_ed_plane(gpl.post, &ep, &it, &ot)) {
					gpl.ed_last = true;
					gpl.off_mid_own = off;
					off += gpl.mid_pitch * gpl.h;
				}
			}
			g->tmp_size = off;
		}
		// GREY to YUV / RGB without a colorspace change: the chroma outputs
		// are the neutral value in the output format, or copies of the luma
		// output (grey_to_yuv / grey_to_rgb, graphbuilder.cpp:615-659)
		if (!colorspace && s.color == COLOR_GREY && d.color != COLOR_GREY) {
			const PixFmt fy = plane_fmt(d, PLANE_Y);
			if (fy.type == ZG_PIXEL_BYTE || fy.type == ZG_PIXEL_WORD)
				g->fill_value = 1u << (fy.depth - 1);
			for (int p : { PLANE_U, PLANE_V }) {
				auto &gpl = g->planes[p];
				gpl.present = gpl.has_dst = true;
				gpl.mode = 7;
				gpl.w = d.planes[p].width;
				gpl.h = d.planes[p].height;
				gpl.out_bytes = bytes(d.pixel_type);
				gpl.dst_ssh = d.color == COLOR_YUV ? d.subsample_h : 0;
				g->out_fill[p] = d.color == COLOR_YUV ? 1 : 2;
			}
		}
		if (colorspace) {
			auto &cm = g->color;
			cm.on = true;
			cm.n_in = s.color == COLOR_GREY ? 1 : 3;
			cm.n_out = d.color == COLOR_GREY ? 1 : 3;
			// work geometry: each dimension from the smaller side
			// (graphbuilder.cpp:982-991)
			const PlaneGeom &sy = s.planes[PLANE_Y], &dy = d.planes[PLANE_Y];
			const PlaneGeom &wsrc = sy.width < dy.width ? sy : dy, &hsrc = sy.height < dy.height ? sy : dy;
			PlaneGeom gw;
			gw.width = wsrc.width;
			gw.left = wsrc.left;
			gw.aw = wsrc.aw;
			gw.height = hsrc.height;
			gw.top = hsrc.top;
			gw.ah = hsrc.ah;
			cm.ww = gw.width;
			cm.wh = gw.height;
			cm.w_pitch = pitch_of(gw.width, 4);
			const bool yuv_in = s.color == COLOR_YUV;
			// after the conversion the planes are YUV unless the output
			// matrix is RGB (convert_colorspace, graphbuilder.cpp:853-861)
			const bool yuv_work = d.cs.m != csp::M_RGB;
			size_t scratch = 0;
			for (int p = 0; p < cm.n_in; ++p) {
				const bool chroma = p != PLANE_Y;
				const int q = (s.color == COLOR_RGB && chroma) ? PLANE_Y : p;
				const bool uv = chroma && yuv_in;
				cm.in[p] = make_chain(s.planes[q], gw, plane_fmt(s, p), PixFmt{ ZG_PIXEL_FLOAT, 32, false, uv },
				                      uv ? gp.resample_filter_uv : gp.resample_filter,
				                      uv ? gp.filter_param_a_uv : gp.filter_param_a,
				                      uv ? gp.filter_param_b_uv : gp.filter_param_b, dither, p);
				scratch = std::max(scratch, cm.in[p].scratch);
				auto &gpl = g->planes[p];
				gpl.present = gpl.has_src = true;
				gpl.mode = 6;
				gpl.in_bytes = bytes(s.pixel_type);
				gpl.src_w = s.planes[q].width;
				gpl.src_h = s.planes[q].height;
				gpl.src_ssh = uv ? s.subsample_h : 0;
			}
			for (int p = 0; p < cm.n_out; ++p) {
				const bool chroma = p != PLANE_Y;
				const int q = (d.color == COLOR_RGB && chroma) ? PLANE_Y : p;
				const bool uv_work = chroma && yuv_work, uv = chroma && d.color == COLOR_YUV;
				cm.out[p] = make_chain(gw, d.planes[q], PixFmt{ ZG_PIXEL_FLOAT, 32, false, uv_work }, plane_fmt(d, p),
				                       uv ? gp.resample_filter_uv : gp.resample_filter,
				                       uv ? gp.filter_param_a_uv : gp.filter_param_a,
				                       uv ? gp.filter_param_b_uv : gp.filter_param_b, dither, p);
				scratch = std::max(scratch, cm.out[p].scratch);
				auto &gpl = g->planes[p];
				gpl.present = gpl.has_dst = true;
				gpl.mode = 6;
				gpl.w = d.planes[q].width;
				gpl.h = d.planes[q].height;
				gpl.out_bytes = bytes(d.pixel_type);
				gpl.dst_ssh = uv ? d.subsample_h : 0;
			}
			// GREY is read as RGB with equal planes (grey_to_rgb before the
			// conversion, graphbuilder.cpp:998-1002)
			csp::Space from = s.cs;
			if (s.color == COLOR_GREY)
				from.m = d.color == COLOR_RGB ? d.cs.m : csp::M_RGB;
			const double peak = std::isnan(gp.nominal_peak_luminance) ? 100.0 : gp.nominal_peak_luminance;
			const bool v25 = gp.version >= ZG_MAKE_API_VERSION(2, 5);
			cm.plan = csp::make_plan(from, d.cs, peak, gp.allow_approximate_gamma != 0,
			                         v25 && gp.scene_referred != 0, v25 && gp.chromatic_adaptation != 0);
			cm.off_work = (g->tmp_size + 255) & ~static_cast<size_t>(255);
			cm.off_scratch = cm.off_work + 3 * cm.w_pitch * cm.wh;
			g->tmp_size = cm.off_scratch + scratch;
		}
		// staging planes for ring buffers, after the largest per-plane scratch
		size_t off = (g->tmp_size + 255) & ~static_cast<size_t>(255);
		for (auto &gpl : g->planes) {
			if (!gpl.present)
				continue;
			gpl.sstage_pitch = pitch_of(gpl.src_w, gpl.in_bytes);
			gpl.off_sstage = off;
			off += gpl.sstage_pitch * gpl.src_h;
			gpl.dstage_pitch = pitch_of(gpl.w, gpl.out_bytes);
			gpl.off_dstage = off;
			off += gpl.dstage_pitch * gpl.h;
		}
		g->tmp_size = off;
		g->src_lines = s.height;
		g->dst_lines = d.height;
		g->src_width = s.width;
		g->dst_width = d.width;
		g->src_step = 1u << s.subsample_h;
		g->dst_step = 1u << d.subsample_h;
		result = g.release();
	});
	return result;
}

void zg_graph_free(zg_graph *g)
{
	delete g;
}

zg_error_code zg_graph_get_tmp_size(const zg_graph *g, size_t *out)
{
	return guarded([&] {
		if (!g || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = g->tmp_size;
	});
}

zg_error_code zg_graph_get_plane_params(const zg_graph *g, int plane, zg_resize_params *out, int *present)
{
	return guarded([&] {
		if (!g || plane < 0 || plane > 3)
			throw Error(kErrIllegalArgument, "bad plane");
		const auto &p = g->planes[plane];
		if (present)
			*present = p.present ? (p.mode == 2 ? 2 : 1) : 0;
		if (out && p.mode == 2)
			*out = p.params;
	});
}

zg_error_code zg_graph_get_input_buffering(const zg_graph *g, unsigned *out)
{
	return guarded([&] {
		if (!g || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = g->src_step;
	});
}

zg_error_code zg_graph_get_output_buffering(const zg_graph *g, unsigned *out)
{
	return guarded([&] {
		if (!g || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = g->dst_step;
	});
}

zg_error_code zg_graph_process(const zg_graph *g, const zg_image_buffer_const *src, const zg_image_buffer *dst,
                               void *tmp, zg_stream stream)
{
	return zg_graph_process_cb(g, src, dst, tmp, nullptr, nullptr, nullptr, nullptr, stream);
}

zg_error_code zg_graph_process_cb(const zg_graph *g, const zg_image_buffer_const *src, const zg_image_buffer *dst,
                                  void *tmp, zg_graph_callback unpack_cb, void *unpack_user, zg_graph_callback pack_cb,
                                  void *pack_user, zg_stream stream)
{
	return guarded([&] {
		if (!g || !src || !dst)
			throw Error(kErrIllegalArgument, "null pointer");
		if (current_device() != g->device)
			throw Error(kErrLogic, "graph used on a different device than the one it was created on");
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		char *t = static_cast<char *>(tmp);
		auto ring_ok = [](unsigned mask) { return mask == ZG_BUFFER_MAX || ((mask + 1) & mask) == 0; };
		// planes' effective source and destination (staging for ring planes)
		const void *from_data[4] = {};
		ptrdiff_t from_stride[4] = {};
		void *to_data[4] = {};
		ptrdiff_t to_stride[4] = {};
		bool src_ring = false, dst_ring = false;
		// ring capacity in luma lines (the smallest ring of the format)
		unsigned src_cap = ~0u, dst_cap = ~0u;
		for (int p = 0; p < 4; ++p) {
			const auto &pl = g->planes[p];
			if (!pl.present)
				continue;
			const unsigned sm = pl.has_src ? src->plane[p].mask : ZG_BUFFER_MAX;
			const unsigned dm = pl.has_dst ? dst->plane[p].mask : ZG_BUFFER_MAX;
			if ((pl.has_src && !src->plane[p].data) || (pl.has_dst && !dst->plane[p].data))
				throw Error(kErrIllegalArgument, "null plane pointer");
			if (!ring_ok(sm) || !ring_ok(dm))
				throw Error(kErrIllegalArgument, "buffer mask must be 2^n - 1 or ZG_BUFFER_MAX");
			if (sm != ZG_BUFFER_MAX) {
				if (((static_cast<unsigned long long>(sm) + 1) << pl.src_ssh) < g->src_step)
					throw Error(kErrIllegalArgument, "input ring buffer smaller than zg_graph_get_input_buffering");
				src_ring = true;
				src_cap = std::min<unsigned long long>(src_cap, (static_cast<unsigned long long>(sm) + 1) << pl.src_ssh);
				if (!t)
					throw Error(kErrIllegalArgument, "tmp is null");
				from_data[p] = t + pl.off_sstage;
				from_stride[p] = static_cast<ptrdiff_t>(pl.sstage_pitch);
			} else if (pl.has_src) {
				from_data[p] = src->plane[p].data;
				from_stride[p] = src->plane[p].stride;
			}
			if (dm != ZG_BUFFER_MAX) {
				if (((static_cast<unsigned long long>(dm) + 1) << pl.dst_ssh) < g->dst_step)
					throw Error(kErrIllegalArgument, "output ring buffer smaller than zg_graph_get_output_buffering");
				dst_ring = true;
				dst_cap = std::min<unsigned long long>(dst_cap, (static_cast<unsigned long long>(dm) + 1) << pl.dst_ssh);
				if (!t)
					throw Error(kErrIllegalArgument, "tmp is null");
				to_data[p] = t + pl.off_dstage;
				to_stride[p] = static_cast<ptrdiff_t>(pl.dstage_pitch);
			} else if (pl.has_dst) {
				to_data[p] = dst->plane[p].data;
				to_stride[p] = dst->plane[p].stride;
			}
		}

		// Input: the unpack callback for each step of lines, as zimg calls it
		// (zimg.h:455-484), and ring lines gathered into whole staging planes
		// before anything reads them. A ring slot is rewritten by the callback
		// only after the copies out of it have completed.
		if (unpack_cb || src_ring) {
			unsigned synced = 0;
			for (unsigned i = 0; i < g->src_lines; i += g->src_step) {
				if (src_ring && i + g->src_step - synced > src_cap) {
					cuda_check(cudaStreamSynchronize(st), "ring buffer copies");
					synced = i;
				}
				if (unpack_cb && unpack_cb(unpack_user, i, 0, g->src_width))
					throw Error(kErrUserCallbackFailed, "user callback failed");
				for (int p = 0; p < 4 && src_ring; ++p) {
					const auto &pl = g->planes[p];
					if (!pl.has_src || src->plane[p].mask == ZG_BUFFER_MAX)
						continue;
					const unsigned l0 = i >> pl.src_ssh;
					const unsigned l1 = std::min(pl.src_h, (i + g->src_step) >> pl.src_ssh);
					for (unsigned l = l0; l < l1; ++l)
						cuda_check(cudaMemcpyAsync(static_cast<char *>(const_cast<void *>(from_data[p])) +
						                               static_cast<ptrdiff_t>(l) * from_stride[p],
						                           static_cast<const char *>(src->plane[p].data) +
						                               static_cast<ptrdiff_t>(l & src->plane[p].mask) * src->plane[p].stride,
						                           static_cast<size_t>(pl.src_w) * pl.in_bytes, cudaMemcpyDeviceToDevice, st),
						           "ring buffer copy");
				}
			}
		}

		struct Deferred {
			const zg_depth *d;
			const void *src;
			ptrdiff_t ss;
			void *dst;
			ptrdiff_t ds;
		};
		std::vector<Deferred> deferred;
		for (int p = 0; p < 4; ++p) {
			const auto &pl = g->planes[p];
			if (!pl.present)
				continue;
			const char *sp = static_cast<const char *>(from_data[p]);
			char *dp = static_cast<char *>(to_data[p]);
			const ptrdiff_t sst = from_stride[p], dst_st = to_stride[p];
			const char *from = sp + static_cast<ptrdiff_t>(pl.off_y) * sst + static_cast<ptrdiff_t>(pl.off_x) * pl.in_bytes;
			if (pl.mode == 0 || pl.mode == 1) {
				copy_plane(dp, dst_st, from, sst, static_cast<size_t>(pl.w) * pl.in_bytes, pl.h, st);
				continue;
			}
			if (pl.mode == 3 || pl.mode == 4) {
				if (pl.ed_last)
					deferred.push_back({ pl.only, from, sst, dp, dst_st });
				else
					run_depth(pl.only, from, sst, dp, dst_st, stream);
				continue;
			}
			if (pl.mode >= 5)
				continue;
			if (pl.tmp && !tmp)
				throw Error(kErrIllegalArgument, "tmp is null");
			const void *rs = sp;
			ptrdiff_t rss = sst;
			if (pl.pre) {
				run_depth(pl.pre, sp, sst, t, static_cast<ptrdiff_t>(pl.pre_pitch), stream);
				rs = t;
				rss = static_cast<ptrdiff_t>(pl.pre_pitch);
			}
			void *rd = pl.post ? static_cast<void *>(t + (pl.ed_last ? pl.off_mid_own : pl.off_mid)) : static_cast<void *>(dp);
			const ptrdiff_t rds = pl.post ? static_cast<ptrdiff_t>(pl.mid_pitch) : dst_st;
			zg_error_code rc = pl.unresize
			                       ? zg_unresize_process(pl.unresize, rs, rss, rd, rds, t ? t + pl.off_tmp : nullptr, stream)
			                       : zg_resize_process(pl.resize, rs, rss, rd, rds, t ? t + pl.off_tmp : nullptr, stream);
			if (rc != ZG_ERROR_SUCCESS) {
				char msg[256];
				zg_get_last_error(msg, sizeof(msg));
				throw Error(rc, msg);
			}
			if (pl.post && pl.ed_last)
				deferred.push_back({ pl.post, rd, rds, dp, dst_st });
			else if (pl.post)
				run_depth(pl.post, rd, rds, dp, dst_st, stream);
		}
		run_ed_planes(deferred.data(), static_cast<int>(deferred.size()), stream);

		if (g->premul.on) {
			const auto &pm = g->premul;
			if (!t)
				throw Error(kErrIllegalArgument, "tmp is null");
			const ptrdiff_t sps = static_cast<ptrdiff_t>(pm.s_pitch), dps = static_cast<ptrdiff_t>(pm.d_pitch);
			auto s_plane = [&](int p) { return t + pm.off_s + static_cast<size_t>(p) * pm.s_pitch * pm.sh; };
			auto d_plane = [&](int p) {
				return pm.across_needed ? t + pm.off_d + static_cast<size_t>(p) * pm.d_pitch * pm.dh : s_plane(p);
			};
			char *rtmp = t + pm.off_rtmp;
			// to FLOAT 4:4:4 at the source luma geometry
			for (int p = 0; p < 4; ++p) {
				if (!g->planes[p].present)
					continue;
				const bool up = (p == PLANE_U || p == PLANE_V) && pm.up;
				if (up) {
					run_depth(pm.in[p], from_data[p], from_stride[p], t + pm.off_cs, static_cast<ptrdiff_t>(pm.cs_pitch),
					          stream);
					run_resize(pm.up, t + pm.off_cs, static_cast<ptrdiff_t>(pm.cs_pitch), s_plane(p), sps, rtmp, stream);
				} else {
					run_depth(pm.in[p], from_data[p], from_stride[p], s_plane(p), sps, stream);
				}
			}
			AlphaLaunch A{};
			A.num_planes = pm.ncolor;
			for (int p = 0; p < pm.ncolor; ++p)
				A.planes[p] = s_plane(p);
			A.stride = sps;
			A.alpha = s_plane(PLANE_A);
			A.alpha_stride = sps;
			A.width = static_cast<int>(pm.sw);
			A.height = static_cast<int>(pm.sh);
			cuda_check(launch_alpha(A, false, st), "premultiply launch");
			if (pm.across_needed) {
				for (int p = 0; p < 4; ++p) {
					if (!g->planes[p].present)
						continue;
					const zg_resize *r = (p == PLANE_U || p == PLANE_V) && pm.across_uv ? pm.across_uv : pm.across;
					run_resize(r, s_plane(p), sps, d_plane(p), dps, rtmp, stream);
				}
			}
			for (int p = 0; p < pm.ncolor; ++p)
				A.planes[p] = d_plane(p);
			A.stride = dps;
			A.alpha = d_plane(PLANE_A);
			A.alpha_stride = dps;
			A.width = static_cast<int>(pm.dw);
			A.height = static_cast<int>(pm.dh);
			cuda_check(launch_alpha(A, true, st), "unpremultiply launch");
			// chroma to its own geometry, then every plane to the output format
			for (int p = 0; p < 4; ++p) {
				if (!g->planes[p].present)
					continue;
				const bool down = (p == PLANE_U || p == PLANE_V) && pm.down;
				if (down) {
					run_resize(pm.down, d_plane(p), dps, t + pm.off_cd, static_cast<ptrdiff_t>(pm.cd_pitch), rtmp, stream);
					run_depth(pm.out[p], t + pm.off_cd, static_cast<ptrdiff_t>(pm.cd_pitch), to_data[p], to_stride[p],
					          stream);
				} else {
					run_depth(pm.out[p], d_plane(p), dps, to_data[p], to_stride[p], stream);
				}
			}
		}

		if (g->color.on) {
			const auto &cm = g->color;
			if (!t)
				throw Error(kErrIllegalArgument, "tmp is null");
			const ptrdiff_t wp = static_cast<ptrdiff_t>(cm.w_pitch);
			auto work = [&](int p) { return t + cm.off_work + static_cast<size_t>(p) * cm.w_pitch * cm.wh; };
			char *scratch = t + cm.off_scratch;
			for (int p = 0; p < cm.n_in; ++p)
				run_chain(cm.in[p], from_data[p], from_stride[p], work(p), wp, scratch, stream);
			for (int p = cm.n_in; p < 3; ++p)
				copy_plane(work(p), wp, work(0), wp, static_cast<size_t>(cm.ww) * 4, cm.wh, st);
			if (cm.plan.num_ops) {
				csp::Launch L{};
				for (int p = 0; p < 3; ++p) {
					L.src[p] = work(p);
					L.dst[p] = work(p);
					L.src_stride[p] = L.dst_stride[p] = wp;
				}
				L.width = static_cast<int>(cm.ww);
				L.height = static_cast<int>(cm.wh);
				L.vec = reinterpret_cast<uintptr_t>(work(0)) % 16 == 0;  // pitches are multiples of 256 bytes
				L.plan = cm.plan;
				cuda_check(csp::launch_colorspace(L, st), "colorspace launch");
			}
			for (int p = 0; p < cm.n_out; ++p)
				run_chain(cm.out[p], work(p), wp, to_data[p], to_stride[p], scratch, stream);
		}
		for (int p = 0; p < 4; ++p) {
			if (g->out_fill[p] == 1) {
				const auto &pl = g->planes[p];
				cuda_check(launch_fill(to_data[p], to_stride[p], static_cast<int>(pl.w), static_cast<int>(pl.h),
				                       static_cast<int>(pl.out_bytes), g->fill_value, st),
				           "plane fill");
			} else if (g->out_fill[p] == 2) {
				const auto &pl = g->planes[p];
				copy_plane(to_data[p], to_stride[p], to_data[PLANE_Y], to_stride[PLANE_Y],
				           static_cast<size_t>(pl.w) * pl.out_bytes, pl.h, st);
			}
		}

		// Output: ring lines scattered from the staging planes a ring's worth
		// at a time, then the pack callback for each step of lines in it, once
		// the copies (and everything before them) have completed.
		if (pack_cb || dst_ring) {
			const unsigned window = dst_ring ? std::max(g->dst_step, dst_cap / g->dst_step * g->dst_step) : g->dst_lines;
			for (unsigned w0 = 0; w0 < g->dst_lines; w0 += window) {
				const unsigned w1 = std::min(g->dst_lines, w0 + window);
				for (int p = 0; p < 4 && dst_ring; ++p) {
					const auto &pl = g->planes[p];
					if (!pl.has_dst || dst->plane[p].mask == ZG_BUFFER_MAX)
						continue;
					const unsigned l0 = w0 >> pl.dst_ssh;
					const unsigned l1 = std::min(pl.h, (w1 + (1u << pl.dst_ssh) - 1) >> pl.dst_ssh);
					for (unsigned l = l0; l < l1; ++l)
						cuda_check(cudaMemcpyAsync(static_cast<char *>(dst->plane[p].data) +
						                               static_cast<ptrdiff_t>(l & dst->plane[p].mask) * dst->plane[p].stride,
						                           static_cast<const char *>(to_data[p]) + static_cast<ptrdiff_t>(l) * to_stride[p],
						                           static_cast<size_t>(pl.w) * pl.out_bytes, cudaMemcpyDeviceToDevice, st),
						           "ring buffer copy");
				}
				cuda_check(cudaStreamSynchronize(st), "ring buffer copies");
				for (unsigned i = w0; i < w1 && pack_cb; i += g->dst_step)
					if (pack_cb(pack_user, i, 0, g->dst_width))
						throw Error(kErrUserCallbackFailed, "user callback failed");
			}
		}
	});
}

} // extern "C"
