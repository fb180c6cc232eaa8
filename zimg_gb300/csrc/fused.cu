// Host planning and launch of the fused two-pass tile kernel.
#include "fused.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace zg {

// per-(H_FIRST, U16) instantiation units (fused_inst_*.cu)
cudaError_t launch_fused_v_f32(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &, cudaStream_t);
cudaError_t launch_fused_v_u16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &, cudaStream_t);
cudaError_t launch_fused_h_f32(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &, cudaStream_t);
cudaError_t launch_fused_h_u16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &, cudaStream_t);
const void *fused_kernel_ptr_v_f32(int hw, int vs);
const void *fused_kernel_ptr_v_u16(int hw, int vs);
const void *fused_kernel_ptr_h_f32(int hw, int vs);
const void *fused_kernel_ptr_h_u16(int hw, int vs);

namespace {

constexpr int kTileW = 128;
constexpr int kHwBuckets[] = { 8, 16 };
constexpr int kVsBuckets[] = { 8, 12, 16, 24 };
constexpr size_t kSmemBudget = 100 * 1024;  // two CTAs per SM at least

int bucket_index(const int *b, int n, int v)
{
	for (int i = 0; i < n; ++i)
		if (v <= b[i])
			return i;
	return -1;
}

size_t align_up(size_t x, size_t a)
{
	return (x + a - 1) / a * a;
}

// u16 sums in float are exact when every partial sum is an integer below 2^24
// and each row's taps sum to exactly 1 << 14 (so re-centring the samples by
// 2^(depth-1) shifts the sum by a multiple of 2^14).
bool u16_exact_in_float(const FilterTable &t, unsigned depth)
{
	const double half = std::ldexp(1.0, static_cast<int>(depth) - 1);
	for (unsigned i = 0; i < t.rows; ++i) {
		double mag = 8192.0;
		long sum = 0;
		for (unsigned k = 0; k < t.width; ++k) {
			const int16_t c = t.i16[static_cast<size_t>(i) * t.width + k];
			mag += std::abs(static_cast<double>(c)) * half;
			sum += c;
		}
		if (sum != 16384 || mag >= 16777216.0)
			return false;
	}
	return true;
}

float tap_value(const FilterTable &t, bool u16, unsigned i, unsigned k)
{
	const size_t at = static_cast<size_t>(i) * t.width + k;
	return u16 ? static_cast<float>(t.i16[at]) : t.f32[at];
}

} // namespace


bool plan_fused(const FilterTable &first, const FilterTable &second, bool h_first, bool u16, unsigned depth,
                unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out)
{
	const FilterTable &H = h_first ? first : second;
	const FilterTable &V = h_first ? second : first;
	if (H.rows != dst_w || V.rows != dst_h || H.input_width != src_w || V.input_width != src_h)
		return false;
	if (u16 && (!u16_exact_in_float(H, depth) || !u16_exact_in_float(V, depth)))
		return false;

	const int hw_i = bucket_index(kHwBuckets, 2, static_cast<int>(H.width));
	if (hw_i < 0)
		return false;
	const int HW = kHwBuckets[hw_i];

	// dense vertical groups
	const unsigned groups = (dst_h + kGroup - 1) / kGroup;
	int max_span = 0;
	std::vector<int> gbase(groups);
	for (unsigned g = 0; g < groups; ++g) {
		int lo = INT_MAX, hi = INT_MIN;
		for (unsigned j = 0; j < kGroup; ++j) {
			const unsigned i = g * kGroup + j;
			if (i >= dst_h)
				break;
			lo = std::min(lo, static_cast<int>(V.left[i]));
			hi = std::max(hi, static_cast<int>(V.left[i] + V.width));
		}
		gbase[g] = lo;
		max_span = std::max(max_span, hi - lo);
	}
	const int vs_i = bucket_index(kVsBuckets, 4, max_span);
	if (vs_i < 0)
		return false;
	const int VS = kVsBuckets[vs_i];

	const int col_align = u16 ? 8 : 4;
	const unsigned tiles_x = (dst_w + kTileW - 1) / kTileW;

	// column windows (shared by all tile heights)
	std::vector<int> win_col(2 * tiles_x);
	int max_px = 0;
	for (unsigned tx = 0; tx < tiles_x; ++tx) {
		int lo = INT_MAX, hi = INT_MIN;
		for (unsigned c = tx * kTileW; c < std::min<unsigned>(dst_w, (tx + 1) * kTileW); ++c) {
			lo = std::min(lo, static_cast<int>(H.left[c]));
			hi = std::max(hi, static_cast<int>(H.left[c]) + HW);
		}
		lo = lo / col_align * col_align;
		win_col[2 * tx] = lo;
		win_col[2 * tx + 1] = hi;
		max_px = std::max(max_px, hi - lo);
	}
	const int pxa = (max_px + 7) & ~7;

	// tile height: as tall as the shared-memory budget allows (a multiple of
	// 16 rows, so each tile's group tables are whole 16-byte chunks)
	int tile_h = h_first ? 64 : 32;
	std::vector<int> win_row;
	size_t smem = 0;
	int max_py = 0;
	for (;; tile_h /= 2) {
		if (tile_h < 16)
			return false;
		const unsigned tiles_y = (dst_h + tile_h - 1) / tile_h;
		win_row.assign(2 * tiles_y, 0);
		max_py = 0;
		for (unsigned ty = 0; ty < tiles_y; ++ty) {
			int lo = INT_MAX, hi = INT_MIN;
			const unsigned g_first = ty * tile_h / kGroup;
			const unsigned g_last = std::min<unsigned>(groups, (ty + 1) * tile_h / kGroup);
			for (unsigned g = g_first; g < g_last; ++g) {
				lo = std::min(lo, gbase[g]);
				hi = std::max(hi, gbase[g] + VS);
			}
			win_row[2 * ty] = lo;
			win_row[2 * ty + 1] = hi;
			max_py = std::max(max_py, hi - lo);
		}
		FusedPlan probe;
		probe.job.h_first = h_first ? 1 : 0;
		probe.job.kind = static_cast<int>(u16 ? FusedKind::U16_EXACT : FusedKind::F32);
		probe.job.tile_h = tile_h;
		probe.job.hw = HW;
		probe.job.vs = VS;
		probe.max_py = max_py;
		probe.max_pitch = pxa + 8;
		const FusedPlan *pp = &probe;
		smem = static_cast<size_t>(fused_layout(&pp, 1).total_bytes);
		if (smem <= kSmemBudget)
			break;
	}
	const unsigned tiles_y = (dst_h + tile_h - 1) / tile_h;
	// The last tile row may hold groups past the plane's last row: they get the
	// last real group's base and zero taps, so every group a tile walks exists.
	const unsigned real_groups = groups;
	const unsigned padded_groups = tiles_y * static_cast<unsigned>(tile_h) / kGroup;
	gbase.resize(padded_groups, gbase[real_groups - 1]);

	// host blob: h_taps | h_left | v_dense | v_base | win_row | win_col
	FusedPlan &p = *out;
	p = FusedPlan{};
	size_t off = 0;
	p.off_h_taps = off;  off = align_up(off + static_cast<size_t>(dst_w) * HW * sizeof(float), 256);
	p.off_h_left = off;  off = align_up(off + static_cast<size_t>(dst_w) * sizeof(int), 256);
	p.off_v_dense = off; off = align_up(off + static_cast<size_t>(padded_groups) * VS * kGroup * sizeof(float), 256);
	p.off_v_base = off;  off = align_up(off + static_cast<size_t>(padded_groups) * sizeof(int), 256);
	p.off_win_row = off; off = align_up(off + win_row.size() * sizeof(int), 256);
	p.off_win_col = off; off = align_up(off + win_col.size() * sizeof(int), 256);
	p.blob.assign(off, 0);

	float *h_taps = reinterpret_cast<float *>(p.blob.data() + p.off_h_taps);
	int *h_left = reinterpret_cast<int *>(p.blob.data() + p.off_h_left);
	for (unsigned c = 0; c < dst_w; ++c) {
		for (unsigned k = 0; k < H.width; ++k)
			h_taps[static_cast<size_t>(c) * HW + k] = tap_value(H, u16, c, k);
		h_left[c] = static_cast<int>(H.left[c]);
	}
	float *v_dense = reinterpret_cast<float *>(p.blob.data() + p.off_v_dense);
	int *v_base = reinterpret_cast<int *>(p.blob.data() + p.off_v_base);
	for (unsigned g = 0; g < padded_groups; ++g) {
		v_base[g] = gbase[g];
		if (g >= real_groups)
			continue;
		for (unsigned j = 0; j < kGroup; ++j) {
			const unsigned i = g * kGroup + j;
			if (i >= dst_h)
				break;
			const int d = static_cast<int>(V.left[i]) - gbase[g];
			for (unsigned k = 0; k < V.width; ++k)
				v_dense[(static_cast<size_t>(g) * VS + d + k) * kGroup + j] = tap_value(V, u16, i, k);
		}
	}
	std::memcpy(p.blob.data() + p.off_win_row, win_row.data(), win_row.size() * sizeof(int));
	std::memcpy(p.blob.data() + p.off_win_col, win_col.data(), win_col.size() * sizeof(int));

	FusedJob &J = p.job;
	J.h_first = h_first ? 1 : 0;
	J.kind = static_cast<int>(u16 ? FusedKind::U16_EXACT : FusedKind::F32);
	J.src_w = static_cast<int>(src_w);
	J.src_h = static_cast<int>(src_h);
	J.dst_w = static_cast<int>(dst_w);
	J.dst_h = static_cast<int>(dst_h);
	J.tile_h = tile_h;
	J.tile_w = kTileW;
	J.tiles_x = static_cast<int>(tiles_x);
	J.tiles_y = static_cast<int>(tiles_y);
	J.hw = HW;
	J.vs = VS;
	const float offset = u16 ? static_cast<float>(std::ldexp(1.0, static_cast<int>(depth) - 1)) : 0.0f;
	J.offset = offset;
	J.magic = 12582912.0f + offset;
	J.pixel_max = u16 ? static_cast<float>((1UL << depth) - 1) : 0.0f;
	p.smem_bytes = smem;
	p.max_py = max_py;
	p.max_pitch = pxa + 8;
	p.variant = ((J.h_first * 2 + (u16 ? 1 : 0)) * 2 + hw_i) * 4 + vs_i;
	return true;
}

void fused_bind(FusedPlan &p, const void *device_blob)
{
	const char *b = static_cast<const char *>(device_blob);
	p.job.h_taps = reinterpret_cast<const float *>(b + p.off_h_taps);
	p.job.h_left = reinterpret_cast<const int *>(b + p.off_h_left);
	p.job.v_dense = reinterpret_cast<const float *>(b + p.off_v_dense);
	p.job.v_base = reinterpret_cast<const int *>(b + p.off_v_base);
	p.job.win_row = reinterpret_cast<const int *>(b + p.off_win_row);
	p.job.win_col = reinterpret_cast<const int *>(b + p.off_win_col);
}

namespace {

void split_variant(int variant, int *hf, int *u16, int *hw_i, int *vs_i)
{
	*vs_i = variant % 4;
	*hw_i = (variant / 4) % 2;
	*u16 = (variant / 8) % 2;
	*hf = (variant / 16) % 2;
}

const void *kernel_ptr(int variant)
{
	int hf, u16, hw, vs;
	split_variant(variant, &hf, &u16, &hw, &vs);
	if (hf)
		return u16 ? fused_kernel_ptr_h_u16(hw, vs) : fused_kernel_ptr_h_f32(hw, vs);
	return u16 ? fused_kernel_ptr_v_u16(hw, vs) : fused_kernel_ptr_v_f32(hw, vs);
}

} // namespace

SmemLayout fused_layout(const FusedPlan *const *plans, int n)
{
	int max_py = 0, max_pitch = 0, max_th = 0, hw = 0, vs = 0;
	bool u16 = false, h_first = false;
	for (int i = 0; i < n; ++i) {
		const FusedPlan &p = *plans[i];
		max_py = std::max(max_py, p.max_py);
		max_pitch = std::max(max_pitch, p.max_pitch);
		max_th = std::max(max_th, p.job.tile_h);
		hw = std::max(hw, p.job.hw);
		vs = std::max(vs, p.job.vs);
		u16 = p.job.kind == static_cast<int>(FusedKind::U16_EXACT);
		h_first = p.job.h_first != 0;
	}
	auto a16 = [](size_t x) { return static_cast<int>((x + 15) / 16 * 16); };
	const int e = u16 ? 2 : 4;
	SmemLayout L{};
	const int patch = a16(static_cast<size_t>(max_py) * max_pitch * e);
	L.vcoef_off = patch;
	L.htaps_off = L.vcoef_off + a16(static_cast<size_t>(max_th / kGroup) * vs * 16);
	L.hleft_off = L.htaps_off + a16(static_cast<size_t>(kTileW) * hw * 4);
	L.vbase_off = L.hleft_off + a16(kTileW * 4);
	L.buf_bytes = L.vbase_off + a16(static_cast<size_t>(max_th / kGroup) * 4);
	L.pf_off = 2 * L.buf_bytes;
	const int pf = u16 ? a16(static_cast<size_t>(max_py) * max_pitch * 4) : 0;
	L.i_off = L.pf_off + pf;
	const size_t ib = h_first ? static_cast<size_t>(max_py) * kTileW * 4 : static_cast<size_t>(max_th) * max_pitch * 4;
	L.total_bytes = L.i_off + a16(ib);
	return L;
}

size_t fused_max_smem()
{
	return kSmemBudget;
}

int fused_grid_size(int variant, size_t smem_bytes)
{
	int dev = 0, sms = 0, per_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const void *k = kernel_ptr(variant);
	cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmemBudget));
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kTileThreads, smem_bytes) != cudaSuccess || per_sm < 1)
		per_sm = 1;
	return std::max(1, sms) * per_sm;
}

cudaError_t launch_fused(int variant, const FusedJob *jobs, int num_jobs, int total_tiles, const SmemLayout &smem_bytes,
                         int grid, const FusedJob &single, cudaStream_t stream)
{
	int hf, u16, hw, vs;
	split_variant(variant, &hf, &u16, &hw, &vs);
	grid = std::max(1, std::min(grid, total_tiles));
	if (hf)
		return u16 ? launch_fused_h_u16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream)
		           : launch_fused_h_f32(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream);
	return u16 ? launch_fused_v_u16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream)
	           : launch_fused_v_f32(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream);
}

void fused_set_io(FusedJob &j, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride)
{
	j.src = src;
	j.src_stride = src_stride;
	j.dst = dst;
	j.dst_stride = dst_stride;
	auto al = [](const void *p, ptrdiff_t s) { return reinterpret_cast<uintptr_t>(p) % 16 == 0 && s % 16 == 0; };
	j.vec_ok = al(src, src_stride) && al(dst, dst_stride) ? 1 : 0;
}

} // namespace zg
