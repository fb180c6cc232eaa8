// Host planning and launch of the tensor-core u16 streaming kernel
// (mma_kernel.cuh), plus its instantiations.
#include "fused.h"
#include "mma_kernel.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace zg {

namespace {

constexpr size_t kMmaSmemMax = 110 * 1024;

size_t align_up(size_t x, size_t a)
{
	return (x + a - 1) / a * a;
}

// IEEE binary16 bits of an integer-valued float that fp16 holds exactly.
uint16_t half_bits(float v)
{
	if (v == 0.0f)
		return std::signbit(v) ? 0x8000 : 0;
	uint32_t u;
	std::memcpy(&u, &v, 4);
	const uint32_t sign = (u >> 16) & 0x8000u;
	const int exp = static_cast<int>((u >> 23) & 0xFF) - 127;
	const uint32_t mant = u & 0x7FFFFFu;
	// exact integers here are normal fp16 numbers (|v| >= 1)
	return static_cast<uint16_t>(sign | static_cast<uint32_t>(exp + 15) << 10 | (mant >> 13));
}

uint32_t pack2(float lo, float hi)
{
	return static_cast<uint32_t>(half_bits(lo)) | (static_cast<uint32_t>(half_bits(hi)) << 16);
}

// The split c = hi + lo with lo = c & 31 (two's complement), hi a multiple of 32.
void split_tap(int16_t c, float *hi, float *lo)
{
	const int l = static_cast<int>(c) & 31;
	*lo = static_cast<float>(l);
	*hi = static_cast<float>(static_cast<int>(c) - l);
}

// 8192 + sum(|hi| + |lo|) * 2^(depth-1) < 2^24 for every output, and each
// row sums to 1 << 14.
bool split_exact(const FilterTable &t, unsigned depth)
{
	const double half = std::ldexp(1.0, static_cast<int>(depth) - 1);
	for (unsigned i = 0; i < t.rows; ++i) {
		double mag = 8192.0;
		long sum = 0;
		for (unsigned k = 0; k < t.width; ++k) {
			float hi, lo;
			const int16_t c = t.i16[static_cast<size_t>(i) * t.width + k];
			split_tap(c, &hi, &lo);
			mag += (std::fabs(hi) + std::fabs(lo)) * half;
			sum += c;
		}
		if (sum != 16384 || mag >= 16777216.0)
			return false;
	}
	return true;
}

int pow2(int x)
{
	int r = 1;
	while (r < x)
		r <<= 1;
	return r;
}

} // namespace

int mma_variant(bool h_first, int kv, int kh)
{
	return 100 + (h_first ? 9 : 0) + (kv - 1) * 3 + (kh - 1);
}

bool plan_mma(const FilterTable &first, const FilterTable &second, bool h_first, unsigned depth, unsigned src_w,
              unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out)
{
	const FilterTable &H = h_first ? first : second;
	const FilterTable &V = h_first ? second : first;
	if (depth > 10 || H.rows != dst_w || V.rows != dst_h || H.input_width != src_w || V.input_width != src_h)
		return false;
	if (!split_exact(H, depth) || !split_exact(V, depth))
		return false;

	// vertical groups of 16 output rows
	const int groups = static_cast<int>((dst_h + 15) / 16);
	std::vector<int> gbase(groups);
	int vspan = 0;
	for (int g = 0; g < groups; ++g) {
		int lo = INT_MAX, hi = INT_MIN;
		for (int r = 0; r < 16; ++r) {
			const unsigned i = static_cast<unsigned>(g * 16 + r);
			if (i >= dst_h)
				break;
			lo = std::min(lo, static_cast<int>(V.left[i]));
			hi = std::max(hi, static_cast<int>(V.left[i] + V.width));
		}
		gbase[g] = lo;
		vspan = std::max(vspan, hi - lo);
		if (g && gbase[g] < gbase[g - 1])
			return false;
	}
	const int KV = (vspan + 15) / 16;
	if (KV < 1 || KV > 3)
		return false;

	// horizontal column groups of 8 outputs, windows aligned down to 8 inputs
	const int cgroups = static_cast<int>((dst_w + 7) / 8);
	std::vector<int> hbase(cgroups);
	int hspan = 0;
	for (int cg = 0; cg < cgroups; ++cg) {
		int lo = INT_MAX, hi = INT_MIN;
		for (int n = 0; n < 8; ++n) {
			const unsigned c = static_cast<unsigned>(cg * 8 + n);
			if (c >= dst_w)
				break;
			lo = std::min(lo, static_cast<int>(H.left[c]));
			hi = std::max(hi, static_cast<int>(H.left[c] + H.width));
		}
		hbase[cg] = lo / 8 * 8;
		hspan = std::max(hspan, hi - hbase[cg]);
	}
	const int KH = (hspan + 15) / 16;
	if (KH < 1 || KH > 3)
		return false;

	// strips: 128 output columns, or 64 when a 128-column strip's rings do not fit
	FusedPlan &p = *out;
	std::vector<int> win_col;
	bool fits = false;
	for (int sw = kStripW; sw >= 64 && !fits; sw /= 2) {
	const int strips = static_cast<int>((dst_w + sw - 1) / sw);
	win_col.assign(2 * strips, 0);
	int max_pxa = 0;
	for (int s = 0; s < strips; ++s) {
		const int cg0 = s * (sw / 8), cg1 = std::min(cgroups, (s + 1) * (sw / 8));
		int lo = INT_MAX, hi = INT_MIN;
		for (int cg = cg0; cg < cg1; ++cg) {
			lo = std::min(lo, hbase[cg]);
			hi = std::max(hi, hbase[cg] + 16 * KH);
		}
		win_col[2 * s] = lo;
		win_col[2 * s + 1] = hi;
		max_pxa = std::max(max_pxa, (hi - lo + 7) & ~7);
	}
	if (h_first && sw != kStripW)
		break;  // intermediate lines are kStripW wide

	// steps, prefetch depth and rings (exact sizes; lines index rings modulo)
	p = FusedPlan{};
	const int step_groups = h_first ? 2 : 1;
	const int nsteps = (groups + step_groups - 1) / step_groups;
	auto hi_of = [&](int k) { return gbase[std::min(groups, (k + 1) * step_groups) - 1] + 16 * KV; };
	// enough source bytes in flight per CTA to cover memory latency
	int new_lines = 1;
	for (int k = 1; k < nsteps; ++k)
		new_lines = std::max(new_lines, hi_of(k) - hi_of(k - 1));
	const int step_bytes = std::max(1, new_lines * max_pxa * 2);
	int ahead = std::max(1, std::min(4, (12 * 1024 + step_bytes - 1) / step_bytes));
	FusedJob &J = p.job;
	for (;; --ahead) {
		int mid_need = 1, src_need = 1, stage_need = 1;
		for (int k = 0; k < nsteps; ++k) {
			const int win_lo = gbase[k * step_groups];
			const int hi = hi_of(k);
			const int hi_ahead = hi_of(std::min(nsteps - 1, k + ahead));
			// 16-line blocks may run up to 15 lines past the step's end
			mid_need = std::max(mid_need, hi - win_lo + 16);
			src_need = std::max(src_need, hi - win_lo + (h_first ? 16 : 0));
			stage_need = std::max(stage_need, hi_ahead - win_lo);
		}
		J.h_first = h_first ? 1 : 0;
		J.kind = static_cast<int>(FusedKind::U16_EXACT);
		J.src_w = static_cast<int>(src_w);
		J.src_h = static_cast<int>(src_h);
		J.dst_w = static_cast<int>(dst_w);
		J.dst_h = static_cast<int>(dst_h);
		J.strips = strips;
		J.strip_w = sw;
		J.groups = groups;
		J.seg_groups = groups;
		J.segments = 1;
		J.step_groups = step_groups;
		J.ring_rows = h_first ? mid_need : 1;
		J.in_rows = src_need;
		J.hw = KH;
		J.vs = KV;
		p.stage_rows = stage_need;
		p.max_pxa = max_pxa;
		p.depth = ahead;
		J.depth = ahead;
		p.mma = true;
		const FusedPlan *pp = &p;
		if (static_cast<size_t>(mma_layout(&pp, 1).total_bytes) <= kMmaSmemMax) {
			fits = true;
			break;
		}
		if (ahead == 1)
			break;
	}
	}
	if (!fits)
		return false;
	FusedJob &J = p.job;

	// tables: hfrag | hbase | vfrag | v_base | win_col
	size_t off = 0;
	p.off_h_taps = off;  off = align_up(off + static_cast<size_t>(cgroups) * KH * 2 * 32 * 8, 256);
	p.off_h_left = off;  off = align_up(off + static_cast<size_t>(cgroups) * 4, 256);
	p.off_v_dense = off; off = align_up(off + static_cast<size_t>(groups) * KV * 2 * 32 * 16, 256);
	p.off_v_base = off;  off = align_up(off + static_cast<size_t>(groups) * 4, 256);
	p.off_win_col = off; off = align_up(off + win_col.size() * 4, 256);
	p.blob.assign(off, 0);

	// B fragments of the horizontal taps: dense [16*KH inputs][8 outputs] per column group
	uint32_t *hfrag = reinterpret_cast<uint32_t *>(p.blob.data() + p.off_h_taps);
	for (int cg = 0; cg < cgroups; ++cg) {
		std::vector<float> dh[2];
		dh[0].assign(16 * KH * 8, 0.0f);
		dh[1].assign(16 * KH * 8, 0.0f);
		for (int n = 0; n < 8; ++n) {
			const unsigned c = static_cast<unsigned>(cg * 8 + n);
			if (c >= dst_w)
				break;
			const int d = static_cast<int>(H.left[c]) - hbase[cg];
			for (unsigned k = 0; k < H.width; ++k) {
				float hi, lo;
				split_tap(H.i16[static_cast<size_t>(c) * H.width + k], &hi, &lo);
				dh[0][(d + k) * 8 + n] = hi;
				dh[1][(d + k) * 8 + n] = lo;
			}
		}
		for (int ks = 0; ks < KH; ++ks)
			for (int h = 0; h < 2; ++h)
				for (int lane = 0; lane < 32; ++lane) {
					const int gid = lane >> 2, tig = lane & 3;
					const int k0 = ks * 16 + 2 * tig;
					uint32_t *f = hfrag + ((static_cast<size_t>(cg) * KH + ks) * 2 + h) * 64 + lane * 2;
					f[0] = pack2(dh[h][k0 * 8 + gid], dh[h][(k0 + 1) * 8 + gid]);
					f[1] = pack2(dh[h][(k0 + 8) * 8 + gid], dh[h][(k0 + 9) * 8 + gid]);
				}
	}
	std::memcpy(p.blob.data() + p.off_h_left, hbase.data(), hbase.size() * 4);

	// A fragments of the vertical taps: dense [16 outputs][16*KV lines] per group
	uint32_t *vfrag = reinterpret_cast<uint32_t *>(p.blob.data() + p.off_v_dense);
	for (int g = 0; g < groups; ++g) {
		std::vector<float> dv[2];
		dv[0].assign(16 * 16 * KV, 0.0f);
		dv[1].assign(16 * 16 * KV, 0.0f);
		const int K = 16 * KV;
		for (int r = 0; r < 16; ++r) {
			const unsigned i = static_cast<unsigned>(g * 16 + r);
			if (i >= dst_h)
				break;
			const int d = static_cast<int>(V.left[i]) - gbase[g];
			for (unsigned k = 0; k < V.width; ++k) {
				float hi, lo;
				split_tap(V.i16[static_cast<size_t>(i) * V.width + k], &hi, &lo);
				dv[0][r * K + d + k] = hi;
				dv[1][r * K + d + k] = lo;
			}
		}
		for (int ks = 0; ks < KV; ++ks)
			for (int h = 0; h < 2; ++h)
				for (int lane = 0; lane < 32; ++lane) {
					const int gid = lane >> 2, tig = lane & 3;
					const int c0 = ks * 16 + 2 * tig;
					uint32_t *f = vfrag + ((static_cast<size_t>(g) * KV + ks) * 2 + h) * 128 + lane * 4;
					const std::vector<float> &a = dv[h];
					f[0] = pack2(a[gid * K + c0], a[gid * K + c0 + 1]);
					f[1] = pack2(a[(gid + 8) * K + c0], a[(gid + 8) * K + c0 + 1]);
					f[2] = pack2(a[gid * K + c0 + 8], a[gid * K + c0 + 9]);
					f[3] = pack2(a[(gid + 8) * K + c0 + 8], a[(gid + 8) * K + c0 + 9]);
				}
	}
	std::memcpy(p.blob.data() + p.off_v_base, gbase.data(), gbase.size() * 4);
	std::memcpy(p.blob.data() + p.off_win_col, win_col.data(), win_col.size() * 4);

	const float offset = static_cast<float>(std::ldexp(1.0, static_cast<int>(depth) - 1));
	J.offset = offset;
	J.magic = 12582912.0f + offset;
	J.pixel_max = static_cast<float>((1UL << depth) - 1);
	p.variant = mma_variant(h_first, KV, KH);
	return true;
}

SmemLayout mma_layout(const FusedPlan *const *plans, int n)
{
	int max_pxa = 0, ring = 1, in = 1, stage = 1, seg_groups = 1, depth = 1, kv = 1, kh = 1, max_sw = 8;
	bool h_first = false;
	for (int i = 0; i < n; ++i) {
		const FusedPlan &p = *plans[i];
		max_sw = std::max(max_sw, p.job.strip_w);
		max_pxa = std::max(max_pxa, p.max_pxa);
		ring = std::max(ring, p.job.ring_rows);
		in = std::max(in, p.job.in_rows);
		stage = std::max(stage, p.stage_rows);
		seg_groups = std::max(seg_groups, p.job.seg_groups);
		depth = std::max(depth, p.depth);
		kv = std::max(kv, p.job.vs);
		kh = std::max(kh, p.job.hw);
		h_first = p.job.h_first != 0;
	}
	auto a16 = [](size_t x) { return static_cast<int>((x + 15) / 16 * 16); };
	SmemLayout L{};
	L.pitch = (max_pxa + 63) / 64 * 64 + 8;  // rows at 16 mod 128 bytes: ldmatrix without bank conflicts
	L.ring_rows = ring;
	L.in_rows = in;
	L.stage_rows = stage;
	L.seg_groups = seg_groups;
	L.step_groups = h_first ? 2 : 1;
	L.depth = depth;
	int off = 0;
	L.ring_off = off;
	off += h_first ? a16(static_cast<size_t>(ring) * mma_detail::kMidPitch * 2) : 0;
	L.stage_off = off;
	off += a16(static_cast<size_t>(stage) * L.pitch * 2);
	L.in_off = off;
	off += a16(static_cast<size_t>(in) * L.pitch * 2);
	L.i_off = off;
	off += h_first ? 0 : a16(static_cast<size_t>(16) * L.pitch * 2);
	L.tile_off = off;                        // staged output rows
	L.tile_pitch = max_sw + 8;
	off += a16(static_cast<size_t>(L.step_groups) * 16 * L.tile_pitch * 2);
	L.htaps_off = off;                       // the strip's horizontal tap fragments
	off += a16(static_cast<size_t>(max_sw / 8) * kh * 2 * 32 * 8);
	L.vcoef_off = off;                       // depth + 1 slots of vertical tap fragments
	off += a16(static_cast<size_t>(depth + 1) * L.step_groups * kv * 2 * 32 * 16);
	L.hleft_off = off;                       // strip column-group bases
	off += a16(static_cast<size_t>(max_sw / 8) * 4);
	L.vbase_off = off;
	off += a16(static_cast<size_t>(seg_groups) * 4);
	L.total_bytes = off;
	return L;
}

namespace {

template <bool HF, int KV, int KH>
const void *mma_ptr()
{
	return reinterpret_cast<const void *>(&mma_detail::mma_kernel<HF, KV, KH>);
}

template <bool HF, int KV>
const void *mma_ptr_kh(int kh)
{
	return kh == 1 ? mma_ptr<HF, KV, 1>() : (kh == 2 ? mma_ptr<HF, KV, 2>() : mma_ptr<HF, KV, 3>());
}

template <bool HF>
const void *mma_ptr_kv(int kv, int kh)
{
	return kv == 1 ? mma_ptr_kh<HF, 1>(kh) : (kv == 2 ? mma_ptr_kh<HF, 2>(kh) : mma_ptr_kh<HF, 3>(kh));
}

} // namespace

const void *mma_kernel_ptr(int variant)
{
	const int v = variant - 100;
	const bool hf = v >= 9;
	const int kv = (v % 9) / 3 + 1, kh = v % 3 + 1;
	return hf ? mma_ptr_kv<true>(kv, kh) : mma_ptr_kv<false>(kv, kh);
}

int mma_threads()
{
	return mma_detail::kThreads;
}

cudaError_t launch_mma(int variant, const FusedJob *jobs, int num_jobs, int total_items, const SmemLayout &L, int grid,
                       const FusedJob &single, cudaStream_t stream)
{
	if (L.total_bytes > static_cast<int>(kMmaSmemMax))
		return cudaErrorInvalidValue;
	const void *k = mma_kernel_ptr(variant);
	cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kMmaSmemMax));
	if (e != cudaSuccess)
		return e;
	FusedJob one = single;
	SmemLayout layout = L;
	void *args[] = { &jobs, &num_jobs, &total_items, &one, &layout };
	grid = std::max(1, std::min(grid, total_items));
	return cudaLaunchKernel(k, dim3(grid), dim3(mma_detail::kThreads), args, static_cast<size_t>(L.total_bytes), stream);
}

} // namespace zg
