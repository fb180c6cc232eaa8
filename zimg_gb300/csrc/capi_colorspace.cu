// C ABI: colorspace conversion objects (zg_colorspace_*), zimg's
// ColorspaceConversion (src/zimg/colorspace/colorspace.cpp:94-121) on three
// device FLOAT planes.
#include <cmath>
#include <cstdint>
#include <string>

#include "capi_common.h"
#include "colorspace_plan.h"

using namespace zg;

struct zg_colorspace {
	int device = 0;
	unsigned width = 0, height = 0;
	csp::Plan plan;
};

extern "C" {

zg_error_code zg_colorspace_create(const zg_colorspace_params *params, zg_colorspace **out)
{
	return guarded([&] {
		if (!params || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = nullptr;
		const zg_colorspace_params &q = *params;
		if (!q.width || !q.height)
			throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
		const csp::Space in = csp::from_api(q.matrix_in, q.transfer_in, q.primaries_in);
		const csp::Space o = csp::from_api(q.matrix_out, q.transfer_out, q.primaries_out);
		// zimg's default peak luminance (colorspace.cpp:84-92)
		const double peak = std::isnan(q.peak_luminance) ? 100.0 : q.peak_luminance;
		auto c = std::make_unique<zg_colorspace>();
		c->width = q.width;
		c->height = q.height;
		c->plan = csp::make_plan(in, o, peak, q.approximate_gamma != 0, q.scene_referred != 0,
		                         q.chromatic_adaptation != 0);
		c->device = current_device();
		*out = c.release();
	});
}

void zg_colorspace_free(zg_colorspace *c)
{
	delete c;
}

zg_error_code zg_colorspace_get_info(const zg_colorspace *c, unsigned *num_ops, int *kinds)
{
	return guarded([&] {
		if (!c || !num_ops)
			throw Error(kErrIllegalArgument, "null pointer");
		*num_ops = static_cast<unsigned>(c->plan.num_ops);
		if (kinds)
			for (int k = 0; k < c->plan.num_ops; ++k)
				kinds[k] = c->plan.ops[k].kind;
	});
}

zg_error_code zg_colorspace_process(const zg_colorspace *c, const void *const src[3], const ptrdiff_t src_stride[3],
                                    void *const dst[3], const ptrdiff_t dst_stride[3], zg_stream stream)
{
	return guarded([&] {
		if (!c || !src || !src_stride || !dst || !dst_stride)
			throw Error(kErrIllegalArgument, "null pointer");
		if (current_device() != c->device)
			throw Error(kErrLogic, "object used on a different device than the one it was created on");
		const ptrdiff_t row = static_cast<ptrdiff_t>(c->width) * 4;
		bool vec = true;
		for (int p = 0; p < 3; ++p) {
			if (!src[p] || !dst[p])
				throw Error(kErrIllegalArgument, "null plane pointer");
			if (abs_stride(src_stride[p]) < row || abs_stride(dst_stride[p]) < row)
				throw Error(kErrIllegalArgument, "stride smaller than a line");
			if (reinterpret_cast<uintptr_t>(src[p]) % 4 || src_stride[p] % 4 || reinterpret_cast<uintptr_t>(dst[p]) % 4 ||
			    dst_stride[p] % 4)
				throw Error(kErrIllegalArgument, "plane not aligned to the sample size");
			vec = vec && reinterpret_cast<uintptr_t>(src[p]) % 16 == 0 && src_stride[p] % 16 == 0 &&
			      reinterpret_cast<uintptr_t>(dst[p]) % 16 == 0 && dst_stride[p] % 16 == 0;
		}
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		if (!c->plan.num_ops) {
			for (int p = 0; p < 3; ++p)
				if (dst[p] != src[p])
					copy_plane(dst[p], dst_stride[p], src[p], src_stride[p], static_cast<size_t>(row), c->height, st);
			return;
		}
		csp::Launch L{};
		for (int p = 0; p < 3; ++p) {
			L.src[p] = src[p];
			L.src_stride[p] = src_stride[p];
			L.dst[p] = dst[p];
			L.dst_stride[p] = dst_stride[p];
		}
		L.width = static_cast<int>(c->width);
		L.height = static_cast<int>(c->height);
		L.vec = vec;
		L.plan = c->plan;
		cuda_check(csp::launch_colorspace(L, st), "colorspace launch");
	});
}

} // extern "C"
