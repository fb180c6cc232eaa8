// C ABI: unresize objects (zg_unresize_*), zimg's UnresizeConversion on
// device planes (src/zimg/unresize/unresize.cpp:34-91).
#include <cstring>
#include <string>

#include "capi_common.h"
#include "unresize.h"

using namespace zg;

namespace {

// A context's tables in one device allocation.
struct DeviceUnresize {
	UnresizeContext ctx;
	DeviceBuffer storage;
	UnresizeTables t{};

	void upload()
	{
		const size_t n = ctx.orig, nc = ctx.coef.size();
		auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
		const size_t o_coef = 0, o_off = up(nc * 4), o_c = o_off + up(n * 4), o_l = o_c + up(n * 4),
		             o_u = o_l + up(n * 4), total = o_u + up(n * 4);
		std::vector<unsigned char> blob(total, 0);
		std::memcpy(blob.data() + o_coef, ctx.coef.data(), nc * 4);
		std::memcpy(blob.data() + o_off, ctx.offset.data(), n * 4);
		std::memcpy(blob.data() + o_c, ctx.lu_c.data(), n * 4);
		std::memcpy(blob.data() + o_l, ctx.lu_l.data(), n * 4);
		std::memcpy(blob.data() + o_u, ctx.lu_u.data(), n * 4);
		storage.reset(total);
		cuda_check(cudaMemcpy(storage.get(), blob.data(), total, cudaMemcpyHostToDevice), "upload unresize tables");
		const char *b = static_cast<const char *>(storage.get());
		t.coef = reinterpret_cast<const float *>(b + o_coef);
		t.offset = reinterpret_cast<const unsigned *>(b + o_off);
		t.lu_c = reinterpret_cast<const float *>(b + o_c);
		t.lu_l = reinterpret_cast<const float *>(b + o_l);
		t.lu_u = reinterpret_cast<const float *>(b + o_u);
		t.up = ctx.up;
		t.orig = ctx.orig;
		t.row_size = ctx.row_size;
	}
};

} // namespace

struct zg_unresize {
	int device = 0;
	zg_unresize_params params{};
	int num_passes = 0;
	bool h_first = false;
	DeviceUnresize h, v;
	ptrdiff_t tmp_stride = 0;
	size_t tmp_size = 0;
};

extern "C" {

zg_error_code zg_unresize_create(const zg_unresize_params *params, zg_unresize **out)
{
	return guarded([&] {
		if (!params || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = nullptr;
		const zg_unresize_params &q = *params;
		if (!q.up_width || !q.up_height || !q.orig_width || !q.orig_height)
			throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
		auto u = std::make_unique<zg_unresize>();
		u->params = q;
		const bool skip_h = q.up_width == q.orig_width && q.shift_w == 0.0;
		const bool skip_v = q.up_height == q.orig_height && q.shift_h == 0.0;
		if (!skip_h && !build_unresize_context(q.orig_width, q.up_width, q.shift_w, &u->h.ctx))
			throw Error(kErrResamplingNotAvailable, "unresize can not upscale");
		if (!skip_v && !build_unresize_context(q.orig_height, q.up_height, q.shift_h, &u->v.ctx))
			throw Error(kErrResamplingNotAvailable, "unresize can not upscale");
		u->num_passes = (skip_h ? 0 : 1) + (skip_v ? 0 : 1);
		u->h_first = skip_v || (!skip_h && unresize_h_first(static_cast<double>(q.orig_width) / q.up_width,
		                                                    static_cast<double>(q.orig_height) / q.up_height));
		if (u->num_passes == 2) {
			// intermediate: orig_width x up_height (H first) or up_width x orig_height
			const unsigned w = u->h_first ? q.orig_width : q.up_width;
			const unsigned h = u->h_first ? q.up_height : q.orig_height;
			u->tmp_stride = static_cast<ptrdiff_t>((static_cast<size_t>(w) * 4 + 255) & ~static_cast<size_t>(255));
			u->tmp_size = static_cast<size_t>(u->tmp_stride) * h;
		}
		u->device = current_device();
		if (!skip_h)
			u->h.upload();
		if (!skip_v)
			u->v.upload();
		*out = u.release();
	});
}

void zg_unresize_free(zg_unresize *u)
{
	delete u;
}

zg_error_code zg_unresize_get_tmp_size(const zg_unresize *u, size_t *out)
{
	return guarded([&] {
		if (!u || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = u->tmp_size;
	});
}

zg_error_code zg_unresize_process(const zg_unresize *u, const void *src, ptrdiff_t src_stride, void *dst,
                                  ptrdiff_t dst_stride, void *tmp, zg_stream stream)
{
	return guarded([&] {
		if (!u)
			throw Error(kErrIllegalArgument, "null pointer");
		if (current_device() != u->device)
			throw Error(kErrLogic, "object used on a different device than the one it was created on");
		const zg_unresize_params &q = u->params;
		auto check = [](const void *p, ptrdiff_t stride, unsigned w, const char *what) {
			if (!p)
				throw Error(kErrIllegalArgument, std::string(what) + " is null");
			if (abs_stride(stride) < static_cast<ptrdiff_t>(w) * 4)
				throw Error(kErrIllegalArgument, std::string(what) + " stride smaller than a line");
			if (reinterpret_cast<uintptr_t>(p) % 4 || stride % 4)
				throw Error(kErrIllegalArgument, std::string(what) + " not aligned to the sample size");
		};
		check(src, src_stride, q.up_width, "src");
		check(dst, dst_stride, q.orig_width, "dst");
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		if (u->num_passes == 0) {
			copy_plane(dst, dst_stride, src, src_stride, static_cast<size_t>(q.up_width) * 4, q.up_height, st);
			return;
		}
		if (u->num_passes == 1) {
			if (u->h_first)
				cuda_check(launch_unresize(u->h.t, true, q.up_height, src, src_stride, dst, dst_stride, st), "unresize");
			else
				cuda_check(launch_unresize(u->v.t, false, q.up_width, src, src_stride, dst, dst_stride, st), "unresize");
			return;
		}
		if (!tmp)
			throw Error(kErrIllegalArgument, "tmp is null");
		if (u->h_first) {
			cuda_check(launch_unresize(u->h.t, true, q.up_height, src, src_stride, tmp, u->tmp_stride, st), "unresize");
			cuda_check(launch_unresize(u->v.t, false, q.orig_width, tmp, u->tmp_stride, dst, dst_stride, st), "unresize");
		} else {
			cuda_check(launch_unresize(u->v.t, false, q.up_width, src, src_stride, tmp, u->tmp_stride, st), "unresize");
			cuda_check(launch_unresize(u->h.t, true, q.orig_height, tmp, u->tmp_stride, dst, dst_stride, st), "unresize");
		}
	});
}

} // extern "C"
