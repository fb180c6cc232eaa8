// Host planning and launch of the chained tensor-core u16 kernel
// (chain_kernel.cuh), plus its instantiations.
#include "chain_kernel.cuh"
#include "fused.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace zg {

namespace {

constexpr size_t kChainSmemMax = 110 * 1024;  // two CTAs per SM
constexpr int kChainKVMax = 3;
constexpr int kChainKHMax = 4;

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
	return static_cast<uint16_t>(sign | static_cast<uint32_t>(exp + 15) << 10 | (mant >> 13));
}

uint32_t pack2(float lo, float hi)
{
	return static_cast<uint32_t>(half_bits(lo)) | (static_cast<uint32_t>(half_bits(hi)) << 16);
}

// c = hi + lo, lo = c & 31 (two's complement), hi a multiple of 32: both exact in fp16.
void split_tap(int16_t c, float *hi, float *lo)
{
	const int l = static_cast<int>(c) & 31;
	*lo = static_cast<float>(l);
	*hi = static_cast<float>(static_cast<int>(c) - l);
}

// 8192 + sum(|hi| + |lo|) * 2^(depth-1) < 2^24 for every output, and each
// row sums to 1 << 14: every fp32 partial sum is an exact integer.
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

// A fragments (m16n8k16, row-major A) of a dense [16][16*K] tap block, hi and
// lo halves: out[((ks * 2 + h) * 32 + lane) * 4 + r].
void a_fragments(const std::vector<float> (&dense)[2], int K, uint32_t *out)
{
	const int W = 16 * K;
	for (int ks = 0; ks < K; ++ks)
		for (int h = 0; h < 2; ++h)
			for (int lane = 0; lane < 32; ++lane) {
				const int gid = lane >> 2, tig = lane & 3;
				const int c0 = ks * 16 + 2 * tig;
				const std::vector<float> &a = dense[h];
				uint32_t *f = out + ((static_cast<size_t>(ks) * 2 + h) * 32 + lane) * 4;
				f[0] = pack2(a[gid * W + c0], a[gid * W + c0 + 1]);
				f[1] = pack2(a[(gid + 8) * W + c0], a[(gid + 8) * W + c0 + 1]);
				f[2] = pack2(a[gid * W + c0 + 8], a[gid * W + c0 + 9]);
				f[3] = pack2(a[(gid + 8) * W + c0 + 8], a[(gid + 8) * W + c0 + 9]);
			}
}

} // namespace

int chain_variant(bool h_first, int kv, int kh)
{
	return 200 + (h_first ? kChainKVMax * kChainKHMax : 0) + (kv - 1) * kChainKHMax + (kh - 1);
}

bool plan_chain(const FilterTable &first, const FilterTable &second, bool h_first, unsigned depth, unsigned src_w,
                unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out)
{
	const FilterTable &H = h_first ? first : second;
	const FilterTable &V = h_first ? second : first;
	if (depth > 10 || H.rows != dst_w || V.rows != dst_h || H.input_width != src_w || V.input_width != src_h)
		return false;
	if (!split_exact(H, depth) || !split_exact(V, depth))
		return false;

	// groups of 16 output rows; window of 16*KV lines from gbase (non-decreasing)
	const int groups = static_cast<int>((dst_h + 15) / 16);
	std::vector<int> gbase(groups);
	int vspan = 0;
	for (int g = 0; g < groups; ++g) {
		int lo = INT_MAX, hi = INT_MIN;
		for (int r = 0; r < 16 && g * 16 + r < static_cast<int>(dst_h); ++r) {
			const unsigned i = static_cast<unsigned>(g * 16 + r);
			lo = std::min(lo, static_cast<int>(V.left[i]));
			hi = std::max(hi, static_cast<int>(V.left[i] + V.width));
		}
		gbase[g] = lo;
		vspan = std::max(vspan, hi - lo);
		if (g && gbase[g] < gbase[g - 1])
			return false;
	}
	const int KV = (vspan + 15) / 16;
	if (KV < 1 || KV > kChainKVMax)
		return false;
	// H first: window starts on multiples of 8 lines where that does not widen
	// the windows past 16 KV lines, so that consecutive groups' windows share
	// whole 8-line blocks, whose horizontal products the kernel keeps
	if (h_first) {
		int vspan8 = 0;
		for (int g = 0; g < groups; ++g) {
			int hi = INT_MIN;
			for (int r = 0; r < 16 && g * 16 + r < static_cast<int>(dst_h); ++r) {
				const unsigned i = static_cast<unsigned>(g * 16 + r);
				hi = std::max(hi, static_cast<int>(V.left[i] + V.width));
			}
			vspan8 = std::max(vspan8, hi - gbase[g] / 8 * 8);
		}
		if ((vspan8 + 15) / 16 == KV)
			for (int g = 0; g < groups; ++g)
				gbase[g] = gbase[g] / 8 * 8;
	}

	// tiles of 16 output columns; window of 16*KH inputs from hstart, which is
	// even (H first: 4-byte fragment loads) or a multiple of 8 (V first: ldmatrix rows)
	const int tiles = static_cast<int>((dst_w + 15) / 16);
	const int align = h_first ? 2 : 8;
	std::vector<int> hstart(tiles);
	int hspan = 0;
	for (int t = 0; t < tiles; ++t) {
		int lo = INT_MAX, hi = INT_MIN;
		for (int n = 0; n < 16 && t * 16 + n < static_cast<int>(dst_w); ++n) {
			const unsigned c = static_cast<unsigned>(t * 16 + n);
			lo = std::min(lo, static_cast<int>(H.left[c]));
			hi = std::max(hi, static_cast<int>(H.left[c] + H.width));
		}
		hstart[t] = lo / align * align;
		hspan = std::max(hspan, hi - hstart[t]);
	}
	const int KH = (hspan + 15) / 16;
	if (KH < 1 || KH > kChainKHMax)
		return false;

	// strips of 8 warps' tiles; source columns [lo, hi) with lo a multiple of 8
	const int strip_tiles = chain_detail::warps_per_cta(h_first) * chain_detail::tiles_per_warp(KV, KH);
	const int strip_w = strip_tiles * chain_detail::kTileW;
	const int strips = static_cast<int>((dst_w + strip_w - 1) / strip_w);
	std::vector<int> win_col(2 * strips);
	int max_pxa = 0;
	for (int s = 0; s < strips; ++s) {
		const int t0 = s * strip_tiles, t1 = std::min(tiles, t0 + strip_tiles);
		int lo = INT_MAX, hi = INT_MIN;
		for (int t = t0; t < t1; ++t) {
			lo = std::min(lo, hstart[t]);
			hi = std::max(hi, hstart[t] + 16 * KH);
		}
		lo = lo / 8 * 8;
		win_col[2 * s] = lo;
		win_col[2 * s + 1] = hi;
		max_pxa = std::max(max_pxa, (hi - lo + 7) & ~7);
	}

	// prefetch depth: about 32 KB of source lines in flight per CTA
	auto hi_of = [&](int g) { return gbase[std::min(g, groups - 1)] + 16 * KV; };
	int new_lines = 1;
	for (int g = 1; g < groups; ++g)
		new_lines = std::max(new_lines, hi_of(g) - hi_of(g - 1));
	const int group_bytes = std::max(1, new_lines * max_pxa * 2);
	FusedPlan &p = *out;
	p = FusedPlan{};
	FusedJob &J = p.job;
	bool fits = false;
	for (int ahead = std::max(1, std::min(8, (32 * 1024 + group_bytes - 1) / group_bytes)); ahead >= 1; --ahead) {
		// a warp may read group g while loads of group g + 1 + ahead land
		int ring = 16 * KV;
		for (int g = 0; g < groups; ++g)
			ring = std::max(ring, hi_of(g + 1 + ahead) - gbase[g]);
		J = FusedJob{};
		J.h_first = h_first ? 1 : 0;
		J.kind = static_cast<int>(FusedKind::U16_EXACT);
		J.src_w = static_cast<int>(src_w);
		J.src_h = static_cast<int>(src_h);
		J.dst_w = static_cast<int>(dst_w);
		J.dst_h = static_cast<int>(dst_h);
		J.strips = strips;
		J.strip_w = strip_w;
		J.groups = groups;
		J.seg_groups = 1;  // work units: (strip, group) pairs, split evenly over the CTAs
		J.segments = groups;
		J.step_groups = 1;
		J.in_rows = ring;
		J.ring_rows = 1;
		J.hw = KH;
		J.vs = KV;
		J.depth = ahead;
		p.max_pxa = max_pxa;
		p.depth = ahead;
		p.mma = true;
		p.chain = true;
		const FusedPlan *pp = &p;
		if (static_cast<size_t>(chain_layout(&pp, 1).total_bytes) <= kChainSmemMax) {
			fits = true;
			break;
		}
	}
	if (!fits)
		return false;

	// tables: h fragments | hstart | v fragments | gbase | win_col
	size_t off = 0;
	p.off_h_taps = off;  off = align_up(off + static_cast<size_t>(tiles) * KH * 2 * 32 * 16, 256);
	p.off_h_left = off;  off = align_up(off + static_cast<size_t>(tiles) * 4, 256);
	p.off_v_dense = off; off = align_up(off + static_cast<size_t>(groups) * KV * 2 * 32 * 16, 256);
	p.off_v_base = off;  off = align_up(off + static_cast<size_t>(groups) * 4, 256);
	p.off_win_col = off; off = align_up(off + win_col.size() * 4, 256);
	p.blob.assign(off, 0);

	// horizontal taps as A: [16 output columns][16*KH inputs from hstart]
	uint32_t *hfrag = reinterpret_cast<uint32_t *>(p.blob.data() + p.off_h_taps);
	for (int t = 0; t < tiles; ++t) {
		std::vector<float> dense[2];
		const int W = 16 * KH;
		dense[0].assign(16 * W, 0.0f);
		dense[1].assign(16 * W, 0.0f);
		for (int n = 0; n < 16 && t * 16 + n < static_cast<int>(dst_w); ++n) {
			const unsigned c = static_cast<unsigned>(t * 16 + n);
			const int d = static_cast<int>(H.left[c]) - hstart[t];
			for (unsigned k = 0; k < H.width; ++k) {
				float hi, lo;
				split_tap(H.i16[static_cast<size_t>(c) * H.width + k], &hi, &lo);
				dense[0][n * W + d + k] = hi;
				dense[1][n * W + d + k] = lo;
			}
		}
		a_fragments(dense, KH, hfrag + static_cast<size_t>(t) * KH * 2 * 32 * 4);
	}
	std::memcpy(p.blob.data() + p.off_h_left, hstart.data(), hstart.size() * 4);

	// vertical taps as A: [16 output rows][16*KV lines from gbase]
	uint32_t *vfrag = reinterpret_cast<uint32_t *>(p.blob.data() + p.off_v_dense);
	for (int g = 0; g < groups; ++g) {
		std::vector<float> dense[2];
		const int W = 16 * KV;
		dense[0].assign(16 * W, 0.0f);
		dense[1].assign(16 * W, 0.0f);
		for (int r = 0; r < 16 && g * 16 + r < static_cast<int>(dst_h); ++r) {
			const unsigned i = static_cast<unsigned>(g * 16 + r);
			const int d = static_cast<int>(V.left[i]) - gbase[g];
			for (unsigned k = 0; k < V.width; ++k) {
				float hi, lo;
				split_tap(V.i16[static_cast<size_t>(i) * V.width + k], &hi, &lo);
				dense[0][r * W + d + k] = hi;
				dense[1][r * W + d + k] = lo;
			}
		}
		a_fragments(dense, KV, vfrag + static_cast<size_t>(g) * KV * 2 * 32 * 4);
	}
	std::memcpy(p.blob.data() + p.off_v_base, gbase.data(), gbase.size() * 4);
	std::memcpy(p.blob.data() + p.off_win_col, win_col.data(), win_col.size() * 4);

	const float offset = static_cast<float>(std::ldexp(1.0, static_cast<int>(depth) - 1));
	J.offset = offset;
	J.magic = 12582912.0f + offset;
	J.pixel_max = static_cast<float>((1UL << depth) - 1);
	p.variant = chain_variant(h_first, KV, KH);
	J.variant = p.variant - 200;
	// H first: the share of a window's 8-line blocks that a group can take
	// over from the previous one (its window moved by a multiple of 8 lines)
	double kept = 0;
	for (int g = 1; g < groups; ++g) {
		const int d = gbase[g] - gbase[g - 1];
		if (h_first && d % 8 == 0 && d / 8 < 2 * KV)
			kept += (2.0 * KV - d / 8) / (2.0 * KV);
	}
	p.reuse_frac = groups > 1 ? static_cast<float>(kept / (groups - 1)) : 0.0f;
	return true;
}

SmemLayout chain_layout(const FusedPlan *const *plans, int n)
{
	int max_pxa = 0, in = 1, seg_groups = 1, depth = 1, kv = 1, tiles = 1;
	for (int i = 0; i < n; ++i) {
		const FusedPlan &p = *plans[i];
		max_pxa = std::max(max_pxa, p.max_pxa);
		in = std::max(in, p.job.in_rows);
		seg_groups = std::max(seg_groups, p.job.groups);  // an item spans up to a whole strip
		depth = std::max(depth, p.depth);
		kv = std::max(kv, p.job.vs);
		tiles = std::max(tiles, chain_detail::tiles_per_warp(p.job.vs, p.job.hw));
	}
	auto a16 = [](size_t x) { return static_cast<int>((x + 15) / 16 * 16); };
	SmemLayout L{};
	// lines at 16 mod 32 bytes: the 8 rows of an ldmatrix phase fall in 8
	// different 16-byte bank groups, and 4-byte fragment loads of 8 lines x 4
	// pairs in 32 different banks
	L.pitch = (max_pxa + 15) / 16 * 16 + 8;
	L.in_rows = in;
	L.ring_rows = 1;
	L.stage_rows = 1;
	L.seg_groups = seg_groups;
	L.step_groups = 1;
	L.depth = depth;
	int off = 0;
	L.in_off = off;
	off += a16(static_cast<size_t>(in) * L.pitch * 2);
	L.vcoef_off = off;
	off += a16(static_cast<size_t>(depth + 2) * kv * 2 * 32 * 16);
	L.tile_off = off;
	L.tile_pitch = chain_detail::kStageBytes / 2;
	off += a16(static_cast<size_t>(chain_detail::kMaxWarps) * tiles * chain_detail::kTileStage);
	L.vbase_off = off;
	off += a16(static_cast<size_t>(seg_groups) * 4);
	L.ring_off = L.stage_off = L.i_off = L.htaps_off = L.hleft_off = off;
	L.total_bytes = off;
	return L;
}

namespace {

template <bool HF, int KV, int KH>
const void *chain_ptr()
{
	return reinterpret_cast<const void *>(&chain_detail::chain_kernel<HF, KV, KH>);
}

template <bool HF, int KV>
const void *chain_ptr_kh(int kh)
{
	switch (kh) {
	case 1: return chain_ptr<HF, KV, 1>();
	case 2: return chain_ptr<HF, KV, 2>();
	case 3: return chain_ptr<HF, KV, 3>();
	default: return chain_ptr<HF, KV, 4>();
	}
}

template <bool HF>
const void *chain_ptr_kv(int kv, int kh)
{
	return kv == 1 ? chain_ptr_kh<HF, 1>(kh) : (kv == 2 ? chain_ptr_kh<HF, 2>(kh) : chain_ptr_kh<HF, 3>(kh));
}

} // namespace

const void *chain_kernel_ptr(int variant)
{
	const int v = variant - 200;
	const int per = kChainKVMax * kChainKHMax;
	const bool hf = v >= per;
	const int kv = (v % per) / kChainKHMax + 1, kh = v % kChainKHMax + 1;
	return hf ? chain_ptr_kv<true>(kv, kh) : chain_ptr_kv<false>(kv, kh);
}

int chain_threads(int variant)
{
	const bool hf = variant - 200 >= kChainKVMax * kChainKHMax;
	return chain_detail::warps_per_cta(hf) * 32;
}

cudaError_t launch_chain(int variant, const FusedJob *jobs, int num_jobs, int total_items, const SmemLayout &L, int grid,
                         const FusedJob &single, cudaStream_t stream)
{
	if (L.total_bytes > static_cast<int>(kChainSmemMax))
		return cudaErrorInvalidValue;
	const void *k = chain_kernel_ptr(variant);
	cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kChainSmemMax));
	if (e != cudaSuccess)
		return e;
	FusedJob one = single;
	SmemLayout layout = L;
	void *args[] = { &jobs, &num_jobs, &total_items, &one, &layout };
	grid = std::max(1, std::min(grid, total_items));
	return cudaLaunchKernel(k, dim3(grid), dim3(chain_threads(variant)), args, static_cast<size_t>(L.total_bytes),
	                        stream);
}

} // namespace zg
