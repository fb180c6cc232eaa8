// Host planning and launch of the fused two-pass tile kernel.
#include "fused.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace zg {

// per-(H_FIRST, kind) instantiation units (fused_inst_*.cu)
cudaError_t launch_fused_v_f32(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
cudaError_t launch_fused_v_u16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
cudaError_t launch_fused_h_f32(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
cudaError_t launch_fused_h_u16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
const void *fused_kernel_ptr_v_f32(int hw, int vs);
const void *fused_kernel_ptr_v_u16(int hw, int vs);
const void *fused_kernel_ptr_h_f32(int hw, int vs);
const void *fused_kernel_ptr_h_u16(int hw, int vs);
cudaError_t launch_fused_v_i16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
cudaError_t launch_fused_h_i16(int, int, const FusedJob *, int, int, const SmemLayout &, int, const FusedJob &,
                               const WorkChunks &, cudaStream_t);
const void *fused_kernel_ptr_v_i16(int hw, int vs);
const void *fused_kernel_ptr_h_i16(int hw, int vs);

namespace {

constexpr int kHwBuckets[] = { 6, 8, 16 };
constexpr int kVsBuckets[] = { 8, 12, 16, 24 };
constexpr size_t kSmemBudget = 56 * 1024;   // preferred: four CTAs of 128 threads per SM
constexpr size_t kSmemMax = 110 * 1024;     // hard limit: two CTAs per SM
constexpr int kItemGroupsMax = 256;          // groups of one work item (a multiple of every step)

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

// zimg's int32 sums cannot overflow: sum |tap| * 2^15 + 8192 < 2^31 per row.
bool u16_fits_int32(const FilterTable &t)
{
	for (unsigned i = 0; i < t.rows; ++i) {
		long long mag = 8192;
		for (unsigned k = 0; k < t.width; ++k)
			mag += static_cast<long long>(std::abs(static_cast<int>(t.i16[static_cast<size_t>(i) * t.width + k]))) << 15;
		if (mag >= (1LL << 31))
			return false;
	}
	return true;
}

// A tap as the kernel reads it: the f32 tap, the int16 tap as a float, or
// (integer arithmetic) the int16 tap as int32 bits.
float tap_value(const FilterTable &t, bool u16, bool integer, unsigned i, unsigned k)
{
	const size_t at = static_cast<size_t>(i) * t.width + k;
	if (integer) {
		const int32_t v = t.i16[at];
		float f;
		std::memcpy(&f, &v, sizeof(f));
		return f;
	}
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
	// u16: exact float arithmetic where the planner can prove it, else zimg's int32
	const bool integer = u16 && (!u16_exact_in_float(H, depth) || !u16_exact_in_float(V, depth));
	if (integer && (!u16_fits_int32(H) || !u16_fits_int32(V)))
		return false;

	const int hw_i = bucket_index(kHwBuckets, 3, static_cast<int>(H.width));
	if (hw_i < 0)
		return false;
	const int HW = kHwBuckets[hw_i];

	// dense vertical groups; streaming needs non-decreasing group bases
	const int kGroup = group_rows(h_first);
	const int groups = static_cast<int>((dst_h + kGroup - 1) / kGroup);
	int max_span = 0;
	std::vector<int> gbase(groups);
	for (int g = 0; g < groups; ++g) {
		int lo = INT_MAX, hi = INT_MIN;
		for (int j = 0; j < kGroup; ++j) {
			const unsigned i = static_cast<unsigned>(g * kGroup + j);
			if (i >= dst_h)
				break;
			lo = std::min(lo, static_cast<int>(V.left[i]));
			hi = std::max(hi, static_cast<int>(V.left[i] + V.width));
		}
		gbase[g] = lo;
		max_span = std::max(max_span, hi - lo);
		if (g && gbase[g] < gbase[g - 1])
			return false;
	}
	const int vs_i = bucket_index(kVsBuckets, 4, max_span);
	if (vs_i < 0)
		return false;
	const int VS = kVsBuckets[vs_i];

	// source-column window of each strip
	const int col_align = u16 ? 8 : 4;
	const int strips = static_cast<int>((dst_w + kStripW - 1) / kStripW);
	std::vector<int> win_col(2 * strips);
	int max_pxa = 0;
	for (int s = 0; s < strips; ++s) {
		int lo = INT_MAX, hi = INT_MIN;
		for (unsigned c = s * kStripW; c < std::min<unsigned>(dst_w, (s + 1) * kStripW); ++c) {
			lo = std::min(lo, static_cast<int>(H.left[c]));
			hi = std::max(hi, static_cast<int>(H.left[c]) + HW);
		}
		lo = lo / col_align * col_align;
		win_col[2 * s] = lo;
		win_col[2 * s + 1] = hi;
		max_pxa = std::max(max_pxa, (hi - lo + 7) & ~7);
	}

	// steps and rings: try the preferred step, then smaller ones
	FusedPlan &p = *out;
	p = FusedPlan{};
	bool fits = false;
	for (int attempt = 0; attempt < 2 && !fits; ++attempt)
	for (int step_groups = 4; step_groups >= 1 && !fits; step_groups /= 2) {
		const size_t budget = attempt == 0 ? kSmemBudget : kSmemMax;
		const int nsteps = (groups + step_groups - 1) / step_groups;
		auto hi_of = [&](int k) { return gbase[std::min(groups, (k + 1) * step_groups) - 1] + VS; };
		int ring_need = 1, stage_need = 1, in_need = 1;
		for (int k = 0; k < nsteps; ++k) {
			const int win_lo = gbase[k * step_groups];
			const int hi = hi_of(k);
			const int hi_next = k + 1 < nsteps ? hi_of(k + 1) : hi;
			// any step may start a segment, when its new lines are its whole window
			if (h_first) {
				ring_need = std::max(ring_need, hi - win_lo);
				if (u16) {
					in_need = std::max(in_need, hi - win_lo);
					stage_need = std::max(stage_need, hi_next - win_lo);
				} else {
					in_need = std::max(in_need, hi_next - win_lo);
				}
			} else {
				ring_need = std::max(ring_need, u16 ? hi - win_lo : hi_next - win_lo);
				if (u16)
					stage_need = std::max(stage_need, hi_next - win_lo);
			}
		}
		auto pow2 = [](int x) { int r = 1; while (r < x) r <<= 1; return r; };
		FusedJob &J = p.job;
		J.h_first = h_first ? 1 : 0;
		J.kind = static_cast<int>(integer ? FusedKind::U16_INT : (u16 ? FusedKind::U16_EXACT : FusedKind::F32));
		J.hw = HW;
		J.vs = VS;
		J.step_groups = step_groups;
		J.groups = groups;
		J.seg_groups = step_groups;  // work units: (strip, step) pairs, split evenly over the CTAs
		J.segments = nsteps;
		J.ring_rows = pow2(ring_need);
		J.in_rows = h_first ? pow2(in_need) : 1;
		p.max_pxa = max_pxa;
		// staging ring for u16 lives in the layout's stage_rows (recorded below)
		p.stage_rows = u16 ? pow2(stage_need) : 1;
		const FusedPlan *pp = &p;
		if (static_cast<size_t>(fused_layout(&pp, 1).total_bytes) <= budget)
			fits = true;
	}
	if (!fits)
		return false;

	// host blob: h_taps | h_left | v_dense | v_base | win_col
	size_t off = 0;
	p.off_h_taps = off;  off = align_up(off + static_cast<size_t>(dst_w) * HW * sizeof(float), 256);
	p.off_h_left = off;  off = align_up(off + static_cast<size_t>(dst_w) * sizeof(int), 256);
	p.off_v_dense = off; off = align_up(off + static_cast<size_t>(groups) * VS * kGroup * sizeof(float), 256);
	p.off_v_base = off;  off = align_up(off + static_cast<size_t>(groups) * sizeof(int), 256);
	p.off_win_col = off; off = align_up(off + win_col.size() * sizeof(int), 256);
	p.blob.assign(off, 0);

	float *h_taps = reinterpret_cast<float *>(p.blob.data() + p.off_h_taps);
	int *h_left = reinterpret_cast<int *>(p.blob.data() + p.off_h_left);
	for (unsigned c = 0; c < dst_w; ++c) {
		for (unsigned k = 0; k < H.width; ++k)
			h_taps[static_cast<size_t>(c) * HW + k] = tap_value(H, u16, integer, c, k);
		h_left[c] = static_cast<int>(H.left[c]);
	}
	float *v_dense = reinterpret_cast<float *>(p.blob.data() + p.off_v_dense);
	int *v_base = reinterpret_cast<int *>(p.blob.data() + p.off_v_base);
	for (int g = 0; g < groups; ++g) {
		v_base[g] = gbase[g];
		for (int j = 0; j < kGroup; ++j) {
			const unsigned i = static_cast<unsigned>(g * kGroup + j);
			if (i >= dst_h)
				break;
			const int d = static_cast<int>(V.left[i]) - gbase[g];
			for (unsigned k = 0; k < V.width; ++k)
				v_dense[(static_cast<size_t>(g) * VS + d + k) * kGroup + j] = tap_value(V, u16, integer, i, k);
		}
	}
	std::memcpy(p.blob.data() + p.off_win_col, win_col.data(), win_col.size() * sizeof(int));

	FusedJob &J = p.job;
	J.src_w = static_cast<int>(src_w);
	J.src_h = static_cast<int>(src_h);
	J.dst_w = static_cast<int>(dst_w);
	J.dst_h = static_cast<int>(dst_h);
	J.strips = strips;
	J.strip_w = kStripW;
	// centring offset: 2^(depth-1) for exact float sums, zimg's 32768 for int32 ones
	const float offset = integer ? 32768.0f : (u16 ? static_cast<float>(std::ldexp(1.0, static_cast<int>(depth) - 1)) : 0.0f);
	J.offset = offset;
	J.magic = 12582912.0f + offset;
	J.pixel_max = u16 ? static_cast<float>((1UL << depth) - 1) : 0.0f;
	p.variant = ((J.h_first * 3 + (integer ? 2 : (u16 ? 1 : 0))) * 3 + hw_i) * 4 + vs_i;
	return true;
}

void fused_segment(FusedPlan *const *plans, int n, int num_items_target)
{
	long strips = 0;
	for (int i = 0; i < n; ++i)
		strips += plans[i]->job.strips;
	const int want = static_cast<int>(std::max<long>(1, (num_items_target + strips - 1) / std::max<long>(1, strips)));
	for (int i = 0; i < n; ++i) {
		FusedJob &J = plans[i]->job;
		if (!plans[i]->mma || plans[i]->chain) {
			// the CUDA-core and chained kernels split their (strip, step)
			// units evenly over their CTAs: one unit per segment
			J.seg_groups = J.step_groups;
			J.segments = (J.groups + J.step_groups - 1) / J.step_groups;
			continue;
		}
		const int steps = (J.groups + J.step_groups - 1) / J.step_groups;
		const int segs = std::max(1, std::min(want, steps));
		const int steps_per_seg = (steps + segs - 1) / segs;
		J.seg_groups = steps_per_seg * J.step_groups;
		J.segments = (J.groups + J.seg_groups - 1) / J.seg_groups;
	}
}

int fused_items(const FusedJob &j)
{
	return j.strips * j.segments;
}

int fused_wave_items()
{
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	return std::max(1, sms) * 4;
}

void fused_bind(FusedPlan &p, const void *device_blob)
{
	const char *b = static_cast<const char *>(device_blob);
	p.job.h_taps = reinterpret_cast<const float *>(b + p.off_h_taps);
	p.job.h_left = reinterpret_cast<const int *>(b + p.off_h_left);
	p.job.v_dense = reinterpret_cast<const float *>(b + p.off_v_dense);
	p.job.v_base = reinterpret_cast<const int *>(b + p.off_v_base);
	p.job.win_col = reinterpret_cast<const int *>(b + p.off_win_col);
}

namespace {

// kind: 0 f32, 1 u16 in exact float sums, 2 u16 in int32 sums
void split_variant(int variant, int *hf, int *kind, int *hw_i, int *vs_i)
{
	*vs_i = variant % 4;
	*hw_i = (variant / 4) % 3;
	*kind = (variant / 12) % 3;
	*hf = (variant / 36) % 2;
}

const void *kernel_ptr(int variant)
{
	if (variant >= 200)
		return chain_kernel_ptr(variant);
	if (variant >= 100)
		return mma_kernel_ptr(variant);
	int hf, kind, hw, vs;
	split_variant(variant, &hf, &kind, &hw, &vs);
	if (hf)
		return kind == 2 ? fused_kernel_ptr_h_i16(hw, vs)
		                 : (kind == 1 ? fused_kernel_ptr_h_u16(hw, vs) : fused_kernel_ptr_h_f32(hw, vs));
	return kind == 2 ? fused_kernel_ptr_v_i16(hw, vs)
	                 : (kind == 1 ? fused_kernel_ptr_v_u16(hw, vs) : fused_kernel_ptr_v_f32(hw, vs));
}

} // namespace

SmemLayout fused_layout(const FusedPlan *const *plans, int n)
{
	if (n > 0 && plans[0]->chain)
		return chain_layout(plans, n);
	if (n > 0 && plans[0]->mma)
		return mma_layout(plans, n);
	int max_pxa = 0, hw = 0, vs = 0, ring = 1, in = 1, stage = 1, seg_groups = 1, step_groups = 1;
	bool u16 = false, h_first = false;
	for (int i = 0; i < n; ++i) {
		const FusedPlan &p = *plans[i];
		max_pxa = std::max(max_pxa, p.max_pxa);
		hw = std::max(hw, p.job.hw);
		vs = std::max(vs, p.job.vs);
		ring = std::max(ring, p.job.ring_rows);
		in = std::max(in, p.job.in_rows);
		stage = std::max(stage, p.stage_rows);
		seg_groups = std::max(seg_groups, std::min(p.job.groups, kItemGroupsMax));
		step_groups = std::max(step_groups, p.job.step_groups);
		u16 = p.job.kind != static_cast<int>(FusedKind::F32);
		h_first = p.job.h_first != 0;
	}
	auto a16 = [](size_t x) { return static_cast<int>((x + 15) / 16 * 16); };
	SmemLayout L{};
	L.pitch = max_pxa + 8;
	L.ring_rows = ring;
	L.in_rows = h_first ? in : 1;
	L.stage_rows = u16 ? stage : 1;
	L.seg_groups = seg_groups;
	L.step_groups = step_groups;
	int off = 0;
	L.ring_off = off;
	off += a16(static_cast<size_t>(ring) * (h_first ? kStripW : L.pitch) * 4);
	L.stage_off = off;
	off += u16 ? a16(static_cast<size_t>(L.stage_rows) * L.pitch * 2) : 0;
	L.in_off = off;
	off += h_first ? a16(static_cast<size_t>(L.in_rows) * L.pitch * 4) : 0;
	L.i_off = off;
	off += h_first ? 0 : a16(static_cast<size_t>(step_groups) * group_rows(false) * L.pitch * 4);
	L.htaps_off = off;
	off += a16(static_cast<size_t>(kStripW) * hw * 4);
	L.hleft_off = off;
	off += a16(kStripW * 4);
	L.vcoef_off = off;
	off += 2 * a16(static_cast<size_t>(step_groups) * vs * group_rows(h_first) * 4);
	L.vbase_off = off;
	off += a16(static_cast<size_t>(seg_groups) * 4);
	L.total_bytes = off;
	return L;
}

size_t fused_max_smem()
{
	return kSmemMax;
}

int fused_grid_size(int variant, size_t smem_bytes)
{
	int dev = 0, sms = 0, per_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const void *k = kernel_ptr(variant);
	cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmemMax));
	const int threads = variant >= 200 ? chain_threads(variant) : (variant >= 100 ? mma_threads() : kStreamThreads);
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem_bytes) != cudaSuccess || per_sm < 1)
		per_sm = 1;
	return std::max(1, sms) * per_sm;
}

bool fused_takes_chunks(int variant)
{
	return variant >= 0 && variant < 100;
}

cudaError_t launch_fused(int variant, const FusedJob *jobs, int num_jobs, int total_tiles, const SmemLayout &smem_bytes,
                         int grid, const FusedJob &single, cudaStream_t stream, const WorkChunks &chunks)
{
	if (variant >= 200)
		return launch_chain(variant, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream);
	if (variant >= 100)
		return launch_mma(variant, jobs, num_jobs, total_tiles, smem_bytes, grid, single, stream);
	int hf, kind, hw, vs;
	split_variant(variant, &hf, &kind, &hw, &vs);
	grid = std::max(1, std::min(grid, total_tiles));
	if (smem_bytes.total_bytes > static_cast<int>(kSmemMax))
		return cudaErrorInvalidValue;
	const WorkChunks &c = chunks;
	if (hf)
		return kind == 2 ? launch_fused_h_i16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream)
		     : kind == 1 ? launch_fused_h_u16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream)
		                 : launch_fused_h_f32(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream);
	return kind == 2 ? launch_fused_v_i16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream)
	     : kind == 1 ? launch_fused_v_u16(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream)
	                 : launch_fused_v_f32(hw, vs, jobs, num_jobs, total_tiles, smem_bytes, grid, single, c, stream);
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
