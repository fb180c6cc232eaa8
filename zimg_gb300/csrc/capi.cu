// C ABI: errors, filter tables, single passes and two-pass conversions.
#include "capi_common.h"

#include <algorithm>
#include <climits>

namespace {

thread_local int g_last_code = ZG_ERROR_SUCCESS;
thread_local std::string g_last_msg;

} // namespace

namespace zg {

void set_last_error(int code, const std::string &msg)
{
	g_last_code = code;
	g_last_msg = msg;
}

Sample sample_of(int pixel_type)
{
	if (pixel_type == ZG_PIXEL_WORD)
		return Sample::U16;
	if (pixel_type == ZG_PIXEL_FLOAT)
		return Sample::F32;
	if (pixel_type == ZG_PIXEL_BYTE || pixel_type == ZG_PIXEL_HALF)
		throw Error(kErrUnsupported, "pixel type not supported by the resize path (WORD or FLOAT)");
	throw Error(kErrEnumOutOfRange, "unrecognized pixel type");
}

unsigned bytes_of(Sample s)
{
	return s == Sample::U16 ? 2 : 4;
}

int current_device()
{
	int d = 0;
	cuda_check(cudaGetDevice(&d), "cudaGetDevice");
	return d;
}

void DevicePass::upload()
{
	const FilterTable &t = table;
	const size_t n = static_cast<size_t>(t.width) * t.rows;
	auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
	const size_t off_f32 = up(t.rows * sizeof(unsigned));
	const size_t off_i16 = off_f32 + up(n * sizeof(float));
	const size_t off_bias = off_i16 + up(n * sizeof(int16_t));
	size_t total = off_bias + up(t.rows * sizeof(int32_t));
	// dense groups of outputs for wide FP32 passes on CUDA cores
	const bool dense = sample == Sample::F32 && t.width >= kDenseTaps;
	const unsigned R = dense_rows(horizontal);
	const unsigned groups = (t.rows + R - 1) / R;
	std::vector<unsigned> dbase(groups), dspan(groups);
	unsigned dstride = 0;  // inputs per group in the dense table (the widest group)
	unsigned dwin = 0;     // widest input window of 32 consecutive groups
	if (dense) {
		for (unsigned g = 0; g < groups; ++g) {
			unsigned lo = ~0u, hi = 0;
			for (unsigned r = 0; r < R && g * R + r < t.rows; ++r) {
				lo = std::min(lo, t.left[g * R + r]);
				hi = std::max(hi, t.left[g * R + r] + t.width);
			}
			dbase[g] = lo;
			dspan[g] = hi - lo;
			dstride = std::max(dstride, dspan[g]);
		}
		for (unsigned g0 = 0; g0 < groups; g0 += 32) {
			unsigned hi = 0;
			for (unsigned g = g0; g < std::min(groups, g0 + 32); ++g)
				hi = std::max(hi, dbase[g] + dspan[g]);
			dwin = std::max(dwin, hi - dbase[g0]);
		}
	}
	const size_t dense_floats = static_cast<size_t>(groups) * dstride * R;
	const size_t off_dbase = total;
	const size_t off_dspan = off_dbase + (dense ? up(groups * sizeof(unsigned)) : 0);
	const size_t off_dense = off_dspan + (dense ? up(groups * sizeof(unsigned)) : 0);
	if (dense)
		total = off_dense + up(dense_floats * sizeof(float));

	std::vector<int32_t> bias(t.rows);
	for (unsigned i = 0; i < t.rows; ++i) {
		int64_t sum = 0;
		for (unsigned k = 0; k < t.width; ++k)
			sum += t.i16[static_cast<size_t>(i) * t.width + k];
		bias[i] = static_cast<int32_t>(static_cast<uint32_t>(static_cast<uint64_t>(-32768 * sum)));
	}

	std::vector<unsigned char> host(total, 0);
	std::memcpy(host.data(), t.left.data(), t.rows * sizeof(unsigned));
	std::memcpy(host.data() + off_f32, t.f32.data(), n * sizeof(float));
	std::memcpy(host.data() + off_i16, t.i16.data(), n * sizeof(int16_t));
	std::memcpy(host.data() + off_bias, bias.data(), t.rows * sizeof(int32_t));
	if (dense) {
		std::memcpy(host.data() + off_dbase, dbase.data(), groups * sizeof(unsigned));
		std::memcpy(host.data() + off_dspan, dspan.data(), groups * sizeof(unsigned));
		float *d = reinterpret_cast<float *>(host.data() + off_dense);
		for (unsigned g = 0; g < groups; ++g)
			for (unsigned r = 0; r < R && g * R + r < t.rows; ++r) {
				const unsigned i = g * R + r;
				for (unsigned k = 0; k < t.width; ++k) {
					const size_t u = t.left[i] - dbase[g] + k;
					const size_t at = horizontal ? (u * groups + g) * R + r : (static_cast<size_t>(g) * dstride + u) * R + r;
					d[at] = t.f32[static_cast<size_t>(i) * t.width + k];
				}
			}
	}

	storage.reset(total);
	cuda_check(cudaMemcpy(storage.get(), host.data(), total, cudaMemcpyHostToDevice), "upload taps");

	unsigned char *base = static_cast<unsigned char *>(storage.get());
	tables.left = reinterpret_cast<const unsigned *>(base);
	tables.f32 = reinterpret_cast<const float *>(base + off_f32);
	tables.i16 = reinterpret_cast<const int16_t *>(base + off_i16);
	tables.bias = reinterpret_cast<const int32_t *>(base + off_bias);
	tables.width = t.width;
	tables.rows = t.rows;
	tables.input_width = t.input_width;
	tables.dense = dense ? reinterpret_cast<const float *>(base + off_dense) : nullptr;
	tables.dbase = dense ? reinterpret_cast<const unsigned *>(base + off_dbase) : nullptr;
	tables.dspan = dense ? reinterpret_cast<const unsigned *>(base + off_dspan) : nullptr;
	tables.dstride = dstride;
	tables.dwin = dwin;
}

void DevicePass::set_tensor()
{
	if (sample != Sample::F32 || wide.frag)
		return;
	std::vector<uint4> frag;
	std::vector<int> kbase;
	int ksteps = 0;
	build_wide_tables(table.f32.data(), table.left.data(), table.width, table.rows, horizontal, &frag, &kbase,
	                  &ksteps);
	std::vector<uint4> uchunk;
	std::vector<int> ubegin, ukbase;
	if (!horizontal)
		build_umma_tables(table.f32.data(), table.left.data(), table.width, table.rows, &uchunk, &ubegin, &ukbase);
	const size_t fbytes = frag.size() * sizeof(uint4);
	const size_t kbytes = kbase.size() * sizeof(int);
	const size_t ubytes = uchunk.size() * sizeof(uint4);
	const size_t bbytes = ubegin.size() * sizeof(int);
	const size_t off_k = fbytes, off_u = (off_k + kbytes + 15) & ~size_t(15), off_b = off_u + ubytes,
	             off_uk = off_b + bbytes;
	wide_storage.reset(off_uk + ukbase.size() * sizeof(int));
	unsigned char *base = static_cast<unsigned char *>(wide_storage.get());
	cuda_check(cudaMemcpy(base, frag.data(), fbytes, cudaMemcpyHostToDevice), "upload band fragments");
	cuda_check(cudaMemcpy(base + off_k, kbase.data(), kbytes, cudaMemcpyHostToDevice), "upload band fragments");
	if (!ukbase.empty()) {
		cuda_check(cudaMemcpy(base + off_u, uchunk.data(), ubytes, cudaMemcpyHostToDevice), "upload band chunks");
		cuda_check(cudaMemcpy(base + off_b, ubegin.data(), bbytes, cudaMemcpyHostToDevice), "upload band chunks");
		cuda_check(cudaMemcpy(base + off_uk, ukbase.data(), ukbase.size() * sizeof(int), cudaMemcpyHostToDevice),
		           "upload band chunks");
	}
	wide.frag = reinterpret_cast<const uint4 *>(base);
	wide.kbase = reinterpret_cast<const int *>(base + off_k);
	wide.groups = static_cast<int>(kbase.size());
	wide.ksteps = ksteps;
	if (!ukbase.empty()) {
		wide.uchunk = reinterpret_cast<const uint4 *>(base + off_u);
		wide.uchunk_begin = reinterpret_cast<const int *>(base + off_b);
		wide.ukbase = reinterpret_cast<const int *>(base + off_uk);
		wide.utiles = static_cast<int>(ukbase.size());
		wide.umax_taps = static_cast<int>(table.width);
	}
}

std::unique_ptr<DevicePass> make_device_pass(const PassSpec &s)
{
	if (!s.src_w || !s.src_h || !s.dst_dim)
		throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
	if (s.sample == Sample::U16 && (s.depth < 1 || s.depth > 16))
		throw Error(kErrBitDepthOverflow, "bit depth exceeds limits of type");

	Kernel k(s.filter, s.a, s.b);
	auto p = std::make_unique<DevicePass>();
	const unsigned src_dim = s.horizontal ? s.src_w : s.src_h;
	p->table = compute_filter(k, src_dim, s.dst_dim, s.shift, default_extent(s.subwidth, src_dim));
	p->horizontal = s.horizontal;
	p->sample = s.sample;
	p->pixel_max = s.sample == Sample::U16 ? static_cast<int32_t>((1UL << s.depth) - 1) : 0;
	p->src_w = s.src_w;
	p->src_h = s.src_h;
	p->dst_w = s.horizontal ? s.dst_dim : s.src_w;
	p->dst_h = s.horizontal ? s.src_h : s.dst_dim;
	p->upload();
	return p;
}

} // namespace zg

using namespace zg;

struct zg_resize_pass {
	int device;
	std::unique_ptr<DevicePass> pass;
};

namespace {

void check_device(int device)
{
	if (current_device() != device)
		throw Error(kErrLogic, "object used on a different device than the one it was created on");
}

void run_pass(const DevicePass &p, const void *src, ptrdiff_t ss, void *dst, ptrdiff_t ds, cudaStream_t stream)
{
	PassLaunch l{};
	l.t = p.tables;
	l.horizontal = p.horizontal;
	l.sample = p.sample;
	l.pixel_max = p.pixel_max;
	l.lines = p.horizontal ? p.src_h : p.src_w;
	l.src = src;
	l.src_stride = ss;
	l.dst = dst;
	l.dst_stride = ds;
	l.wide = p.wide;
	cuda_check(launch_pass(l, stream), "resize pass launch");
}

void check_plane(const void *p, ptrdiff_t stride, unsigned w, Sample s, const char *what)
{
	if (!p)
		throw Error(kErrIllegalArgument, std::string(what) + " is null");
	if (abs_stride(stride) < static_cast<ptrdiff_t>(w) * static_cast<ptrdiff_t>(bytes_of(s)))
		throw Error(kErrIllegalArgument, std::string(what) + " stride smaller than a line");
	if (reinterpret_cast<uintptr_t>(p) % bytes_of(s) || stride % bytes_of(s))
		throw Error(kErrIllegalArgument, std::string(what) + " not aligned to the sample size");
}

} // namespace


extern "C" {

int zg_wide_forms_used(int reset)
{
	return wide_forms_used(reset != 0);
}

int zg_pipeline_status(int reset)
{
	const int chain = chain_tma_pipeline_error(reset != 0);
	const int wide = wide_umma_pipeline_error(reset != 0);
	if (chain < 0 || wide < 0)
		return -1;
	return (chain & 0xFF) | (wide ? (16 + wide) << 8 : 0);
}

int zg_debug_pipeline_fault(int drop_group, unsigned long long wait_ns)
{
	return chain_tma_set_fault(drop_group, wait_ns);
}

zg_error_code zg_get_last_error(char *err_msg, size_t n)
{
	if (err_msg && n) {
		std::strncpy(err_msg, g_last_msg.c_str(), n - 1);
		err_msg[n - 1] = '\0';
	}
	return static_cast<zg_error_code>(g_last_code);
}

void zg_clear_last_error(void)
{
	g_last_code = ZG_ERROR_SUCCESS;
	g_last_msg.clear();
}

void zg_get_version_info(unsigned *major, unsigned *minor, unsigned *micro)
{
	if (major) *major = ZG_API_VERSION_MAJOR;
	if (minor) *minor = ZG_API_VERSION_MINOR;
	if (micro) *micro = 0;
}

zg_error_code zg_compute_filter(zg_resample_filter filter, double param_a, double param_b, unsigned src_dim,
                                unsigned dst_dim, double shift, double width, unsigned *filter_width,
                                unsigned *filter_rows, float *f32, int16_t *i16, unsigned *left)
{
	return guarded([&] {
		if (!filter_width || !filter_rows)
			throw Error(kErrIllegalArgument, "null output pointer");
		Kernel k(filter, param_a, param_b);
		FilterTable t = compute_filter(k, src_dim, dst_dim, shift, default_extent(width, src_dim));
		*filter_width = t.width;
		*filter_rows = t.rows;
		if (f32) {
			if (!i16 || !left)
				throw Error(kErrIllegalArgument, "null output pointer");
			std::memcpy(f32, t.f32.data(), t.f32.size() * sizeof(float));
			std::memcpy(i16, t.i16.data(), t.i16.size() * sizeof(int16_t));
			std::memcpy(left, t.left.data(), t.left.size() * sizeof(unsigned));
		}
	});
}

zg_error_code zg_resize_pass_create(const zg_pass_params *params, zg_resize_pass **out)
{
	return guarded([&] {
		if (!params || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = nullptr;
		PassSpec s{ params->src_width, params->src_height, sample_of(params->pixel_type), params->depth,
		            params->horizontal != 0, params->dst_dim, params->filter, params->filter_param_a,
		            params->filter_param_b, params->shift, params->subwidth };
		auto r = std::make_unique<zg_resize_pass>();
		r->device = current_device();
		r->pass = make_device_pass(s);
		*out = r.release();
	});
}

void zg_resize_pass_free(zg_resize_pass *pass)
{
	delete pass;
}

zg_error_code zg_resize_pass_get_output(const zg_resize_pass *pass, unsigned *width, unsigned *height)
{
	return guarded([&] {
		if (!pass)
			throw Error(kErrIllegalArgument, "null pointer");
		if (width) *width = pass->pass->dst_w;
		if (height) *height = pass->pass->dst_h;
	});
}

zg_error_code zg_resize_pass_process(const zg_resize_pass *pass, const void *src, ptrdiff_t src_stride, void *dst,
                                     ptrdiff_t dst_stride, zg_stream stream)
{
	return guarded([&] {
		if (!pass)
			throw Error(kErrIllegalArgument, "null pointer");
		check_device(pass->device);
		const DevicePass &p = *pass->pass;
		check_plane(src, src_stride, p.src_w, p.sample, "src");
		check_plane(dst, dst_stride, p.dst_w, p.sample, "dst");
		run_pass(p, src, src_stride, dst, dst_stride, reinterpret_cast<cudaStream_t>(stream));
	});
}

void zg_resize_params_default(zg_resize_params *p)
{
	if (!p)
		return;
	std::memset(p, 0, sizeof(*p));
	p->pixel_type = ZG_PIXEL_FLOAT;
	p->depth = 32;
	p->filter = ZG_RESIZE_BICUBIC;
	p->filter_param_a = NAN;
	p->filter_param_b = NAN;
	p->subwidth = NAN;
	p->subheight = NAN;
	p->engine = ZG_ENGINE_AUTO;
	p->allow_fusion = 1;
}

zg_error_code zg_resize_create(const zg_resize_params *params, zg_resize **out)
{
	return guarded([&] {
		if (!params || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = nullptr;
		const zg_resize_params &q = *params;
		if (!q.src_width || !q.src_height || !q.dst_width || !q.dst_height)
			throw Error(kErrInvalidImageSize, "image dimensions must be non-zero");
		auto r = std::make_unique<zg_resize>();
		r->device = current_device();
		r->params = q;
		r->sample = sample_of(q.pixel_type);
		const double subw = default_extent(q.subwidth, q.src_width);
		const double subh = default_extent(q.subheight, q.src_height);
		r->params.subwidth = subw;
		r->params.subheight = subh;
		if (r->sample == Sample::U16 && (q.depth < 1 || q.depth > 16))
			throw Error(kErrBitDepthOverflow, "bit depth exceeds limits of type");
		// Kernel construction validates the filter even when no pass is needed.
		Kernel probe(q.filter, q.filter_param_a, q.filter_param_b);
		(void)probe;

		bool order[2] = { false, false };
		r->num_passes = plan_pass_order(q.src_width, q.src_height, q.dst_width, q.dst_height, q.shift_w, q.shift_h,
		                                subw, subh, order);
		r->first_horizontal = r->num_passes ? order[0] : false;

		unsigned cur_w = q.src_width, cur_h = q.src_height;
		for (int p = 0; p < r->num_passes; ++p) {
			const bool h = order[p];
			PassSpec s{ cur_w, cur_h, r->sample, q.depth, h, h ? q.dst_width : q.dst_height, q.filter,
			            q.filter_param_a, q.filter_param_b, h ? q.shift_w : q.shift_h, h ? subw : subh };
			r->pass[p] = make_device_pass(s);
			cur_w = r->pass[p]->dst_w;
			cur_h = r->pass[p]->dst_h;
		}
		if (r->num_passes == 2) {
			const DevicePass &p0 = *r->pass[0];
			r->tmp_stride = static_cast<ptrdiff_t>((static_cast<size_t>(p0.dst_w) * bytes_of(r->sample) + 255) & ~static_cast<size_t>(255));
			r->tmp_size = static_cast<size_t>(r->tmp_stride) * p0.dst_h;
			const bool u16 = r->sample == Sample::U16;
			bool planned = false;
			if (q.allow_fusion && u16 && q.engine != ZG_ENGINE_CUDA)
				planned = plan_chain(r->pass[0]->table, r->pass[1]->table, r->first_horizontal, q.depth, q.src_width,
				                     q.src_height, q.dst_width, q.dst_height, &r->fplan);
			if (!planned && q.allow_fusion && u16 && q.engine != ZG_ENGINE_CUDA)
				planned = plan_mma(r->pass[0]->table, r->pass[1]->table, r->first_horizontal, q.depth, q.src_width,
				                   q.src_height, q.dst_width, q.dst_height, &r->fplan);
			if (!planned && q.allow_fusion && q.engine != ZG_ENGINE_TENSOR)
				planned = plan_fused(r->pass[0]->table, r->pass[1]->table, r->first_horizontal, u16, q.depth,
				                     q.src_width, q.src_height, q.dst_width, q.dst_height, &r->fplan);
			if (planned) {
				r->fblob.reset(r->fplan.blob.size());
				cuda_check(cudaMemcpy(r->fblob.get(), r->fplan.blob.data(), r->fplan.blob.size(),
				                      cudaMemcpyHostToDevice), "upload fused tables");
				fused_bind(r->fplan, r->fblob.get());
				FusedPlan *mp = &r->fplan;
				fused_segment(&mp, 1, fused_wave_items());
				const FusedPlan *pp = &r->fplan;
				r->flayout = fused_layout(&pp, 1);
				r->fgrid = fused_grid_size(r->fplan.variant, static_cast<size_t>(r->flayout.total_bytes));
				if (r->fplan.chain && chain_tma_enabled()) {
					r->tma = chain_tma_layout(&pp, 1, &r->tlayout);
					if (r->tma)
						r->tgrid = chain_tma_grid_size(r->fplan.variant, static_cast<size_t>(r->tlayout.total_bytes));
				}
				r->fused = true;
				r->tmp_size = 0;
			}
		}
		if (!r->fused && r->sample == Sample::F32 && q.engine != ZG_ENGINE_CUDA) {
			// unfused FP32 passes: wide filters (or an explicit request) on the tensor cores
			for (int p = 0; p < r->num_passes; ++p) {
				if (q.engine == ZG_ENGINE_TENSOR || r->pass[p]->table.width >= kWideTaps) {
					r->pass[p]->set_tensor();
					r->tensor_passes = true;
				}
			}
		}
		*out = r.release();
	});
}

void zg_resize_free(zg_resize *r)
{
	delete r;
}

zg_error_code zg_resize_get_tmp_size(const zg_resize *r, size_t *out)
{
	return guarded([&] {
		if (!r || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = r->tmp_size;
	});
}

zg_error_code zg_resize_get_info(const zg_resize *r, int *num_passes, int *first_horizontal, int *fused)
{
	return guarded([&] {
		if (!r)
			throw Error(kErrIllegalArgument, "null pointer");
		if (num_passes) *num_passes = r->num_passes;
		if (first_horizontal) *first_horizontal = r->first_horizontal;
		if (fused) *fused = r->fused ? (r->fplan.mma ? 2 : 1) : (r->tensor_passes ? 3 : 0);
	});
}

zg_error_code zg_resize_process(const zg_resize *r, const void *src, ptrdiff_t src_stride, void *dst,
                                ptrdiff_t dst_stride, void *tmp, zg_stream stream)
{
	return guarded([&] {
		if (!r)
			throw Error(kErrIllegalArgument, "null pointer");
		check_device(r->device);
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		const zg_resize_params &q = r->params;
		check_plane(src, src_stride, q.src_width, r->sample, "src");
		check_plane(dst, dst_stride, q.dst_width, r->sample, "dst");
		if (r->num_passes == 0) {
			copy_plane(dst, dst_stride, src, src_stride, static_cast<size_t>(q.dst_width) * bytes_of(r->sample),
			           q.dst_height, st);
			return;
		}
		if (r->num_passes == 1) {
			run_pass(*r->pass[0], src, src_stride, dst, dst_stride, st);
			return;
		}
		if (r->fused) {
			FusedJob j = r->fplan.job;
			fused_set_io(j, src, src_stride, dst, dst_stride);
			j.item_begin = 0;
			CUtensorMap map;
			if (r->tma && chain_tma_source_map(&map, j, r->tlayout)) {
				cuda_check(launch_chain_tma(r->fplan.variant, nullptr, 1, fused_items(j), nullptr, r->tlayout, r->tgrid, j, &map,
				                            st),
				           "fused resize launch");
				return;
			}
			cuda_check(launch_fused(r->fplan.variant, nullptr, 1, fused_items(j), r->flayout, r->fgrid,
			                        j, st), "fused resize launch");
			return;
		}
		if (!tmp)
			throw Error(kErrIllegalArgument, "tmp buffer required (zg_resize_get_tmp_size)");
		if (reinterpret_cast<uintptr_t>(tmp) % 256)
			throw Error(kErrIllegalArgument, "tmp buffer must be 256-byte aligned");
		run_pass(*r->pass[0], src, src_stride, tmp, r->tmp_stride, st);
		run_pass(*r->pass[1], tmp, r->tmp_stride, dst, dst_stride, st);
	});
}

} // extern "C"
