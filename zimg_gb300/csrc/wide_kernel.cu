// FP32 resize passes with wide filters (strong downscales: tens to hundreds
// of taps per output) as banded matrix products on the tensor cores.
//
// One pass computes out[o][m] = sum_k tap(o, k) * in[k][m] for every output
// o along the filtered axis and every m across it (m = column for a vertical
// pass, row for a horizontal one). Outputs are taken 8 at a time; over the
// inputs its 8 outputs touch, a group's taps form a dense 8 x K block, so the
// pass is a sequence of small GEMMs D[16 m][8 o] += A[16 m][8 k] * B[8 k][8 o]
// (mma.sync m16n8k8, tf32 operands, fp32 accumulation).
//
// Precision (3xTF32): every f32 operand x is split into x_hi = tf32(x) and
// x_lo = tf32(x - x_hi); each product is a_hi*b_hi + a_hi*b_lo + a_lo*b_hi,
// which keeps about 21 significant bits of every tap * sample product. The
// taps are zimg's f32 taps (filter.cpp:43-127), so the kernel approximates
// the same sums as the C path's resize_line_{h,v}_f32_c
// (resize_impl.cpp:61-114), summed in a different order.
//
// Fragment layouts follow the PTX ISA description of mma.m16n8k8 (.tf32):
// groupID = lane >> 2, tig = lane & 3;
//   A: a0 (gid, tig), a1 (gid + 8, tig), a2 (gid, tig + 4), a3 (gid + 8, tig + 4)
//   B: b0 (k = tig, n = gid), b1 (k = tig + 4, n = gid)
//   D: d0 (gid, 2 tig), d1 (gid, 2 tig + 1), d2 (gid + 8, 2 tig), d3 (gid + 8, 2 tig + 1)
//
// Inputs of a group's block that lie outside an output's band get zero taps;
// they are still read (clamped to the plane), so a non-finite sample within
// a group's block reaches the group's other outputs as NaN.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "kernels.h"

namespace zg {

namespace {

constexpr int kWideWarps = 4;

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
	asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
	             "{%8, %9}, {%0, %1, %2, %3};\n"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t tf32_rna(float x)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return r;
}

// One k-step: 4 samples of this lane -> split -> three products.
__device__ __forceinline__ void step3(float (&d)[4], float x0, float x1, float x2, float x3, const uint4 &b)
{
	const uint32_t h0 = tf32_rna(x0), h1 = tf32_rna(x1), h2 = tf32_rna(x2), h3 = tf32_rna(x3);
	const uint32_t l0 = tf32_rna(x0 - __uint_as_float(h0));
	const uint32_t l1 = tf32_rna(x1 - __uint_as_float(h1));
	const uint32_t l2 = tf32_rna(x2 - __uint_as_float(h2));
	const uint32_t l3 = tf32_rna(x3 - __uint_as_float(h3));
	mma_tf32(d, l0, l1, l2, l3, b.x, b.y);
	mma_tf32(d, h0, h1, h2, h3, b.z, b.w);
	mma_tf32(d, h0, h1, h2, h3, b.x, b.y);
}

// One accumulator carried through all k-steps of a 600-tap band (about 160
// k-steps) measured 7x the C path's error against FP64: the tensor cores'
// fp32 additions are not IEEE round-to-nearest. Chunks of at most 4 k-steps
// start from zero and are added to the running sum with ordinary fp32 adds.
__device__ __forceinline__ void add4(float (&d)[4], const float (&c)[4])
{
	d[0] += c[0];
	d[1] += c[1];
	d[2] += c[2];
	d[3] += c[3];
}

// Ask L2 for the source rows of k-steps [s, s + 4) of this warp's tile (pf:
// the tile's first line; PERM_K: lines m0 + lane % 16 from input kb + 8 s,
// both 64-byte halves of the 128 bytes; otherwise inputs kb + 8 s + lane,
// the tile's 64 bytes of columns): one instruction per 4 k-steps.
template <bool PERM_K>
__device__ __forceinline__ void prefetch4(const char *pf, int kb, int s, int src_dim, int m_left, ptrdiff_t sm,
                                          ptrdiff_t sk)
{
	const int lane = threadIdx.x & 31;
	const char *a;
	if (PERM_K) {
		if ((lane & 15) >= m_left || kb + 8 * s + 16 * (lane >> 4) >= src_dim)
			return;
		a = pf + (lane & 15) * sm + static_cast<ptrdiff_t>(kb + 8 * s) * sk + (lane >> 4) * 64;
	} else {
		if (kb + 8 * s + lane >= src_dim)
			return;
		a = pf + static_cast<ptrdiff_t>(kb + 8 * s + lane) * sk;
	}
	asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a));
}

constexpr int kPrefetchSteps = 16;  // k-steps between a prefetch and the loads it serves

// k-steps [s0, s1) of output group g for this lane's rows/columns ma, mb:
// d += sum of the 3xTF32 products. Element (m, k) of the input is at
// src + m * sm + k * sk (bytes).
//
// Fragment index maps (the B fragments are built to match, build_wide_tables):
//   PERM_K (horizontal passes): k = tig reads input kb + 8s + 2 tig and
//     k = tig + 4 reads the next sample, so each lane's pair is adjacent;
//   otherwise k = tig and tig + 4 read inputs kb + 8s + tig and + tig + 4.
// PAIR: the lane's two samples of a k-step lie 4 bytes apart (ma, mb adjacent
// columns in a vertical pass, or the PERM_K pair) and the plane is 8-byte
// aligned: one 8-byte load each.
// pf, m_left (lines from the tile's first to the plane's end), sm: the
// prefetch of the rows kPrefetchSteps ahead (prefetch4).
template <bool PERM_K, bool PAIR>
__device__ __forceinline__ void band_sum(float (&d)[4], const WideTables &w, int g, int s0, int s1, int src_dim,
                                         const char *base_a, const char *base_b, ptrdiff_t sk, const char *pf,
                                         int m_left, ptrdiff_t sm)
{
	const int lane = threadIdx.x & 31, tig = lane & 3;
	const int kb = __ldg(w.kbase + g);
	const uint4 *bf = w.frag + static_cast<size_t>(g) * w.ksteps * 32 + lane;
	const int koff = PERM_K ? 2 * tig : tig;        // this lane's k = tig input
	const ptrdiff_t khi = PERM_K ? sk : 4 * sk;     // k = tig + 4 relative to k = tig
	if (kb + 8 * s1 <= src_dim) {
		const char *pa = base_a + (kb + 8 * s0 + koff) * sk, *pb = base_b + (kb + 8 * s0 + koff) * sk;
		const ptrdiff_t s8 = 8 * sk;
		// chunks of 4 k-steps, double-buffered: the loads of the next chunk are
		// in flight while the current one runs on the tensor cores
		auto load4 = [&](float (&x)[4][4], uint4 (&b)[4], int s) {
			const char *qa = pa + static_cast<ptrdiff_t>(s - s0) * s8, *qb = pb + static_cast<ptrdiff_t>(s - s0) * s8;
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				if (PAIR && PERM_K) {
					// (k = tig, k = tig + 4) of rows ma and mb
					const float2 va = __ldg(reinterpret_cast<const float2 *>(qa + u * s8));
					const float2 vb = __ldg(reinterpret_cast<const float2 *>(qb + u * s8));
					x[u][0] = va.x;
					x[u][2] = va.y;
					x[u][1] = vb.x;
					x[u][3] = vb.y;
				} else if (PAIR) {
					// columns ma, mb = ma + 1 of lines k = tig and tig + 4
					const float2 v0 = __ldg(reinterpret_cast<const float2 *>(qa + u * s8));
					const float2 v1 = __ldg(reinterpret_cast<const float2 *>(qa + u * s8 + khi));
					x[u][0] = v0.x;
					x[u][1] = v0.y;
					x[u][2] = v1.x;
					x[u][3] = v1.y;
				} else {
					x[u][0] = __ldg(reinterpret_cast<const float *>(qa + u * s8));
					x[u][1] = __ldg(reinterpret_cast<const float *>(qb + u * s8));
					x[u][2] = __ldg(reinterpret_cast<const float *>(qa + u * s8 + khi));
					x[u][3] = __ldg(reinterpret_cast<const float *>(qb + u * s8 + khi));
				}
				b[u] = __ldg(bf + (s + u) * 32);
			}
		};
		auto run4 = [&](const float (&x)[4][4], const uint4 (&b)[4]) {
			float c[4] = { 0.f, 0.f, 0.f, 0.f };
#pragma unroll
			for (int u = 0; u < 4; ++u)
				step3(c, x[u][0], x[u][1], x[u][2], x[u][3], b[u]);
			add4(d, c);
		};
		int s = s0;
		if (s + 4 <= s1) {
			float xa[4][4], xb[4][4];
			uint4 ba[4], bb[4];
			load4(xa, ba, s);
			for (;;) {
				const bool has_b = s + 8 <= s1;
				prefetch4<PERM_K>(pf, kb, s + kPrefetchSteps, src_dim, m_left, sm, sk);
				if (has_b)
					load4(xb, bb, s + 4);
				run4(xa, ba);
				s += 4;
				if (!has_b)
					break;
				const bool has_a = s + 8 <= s1;
				prefetch4<PERM_K>(pf, kb, s + kPrefetchSteps, src_dim, m_left, sm, sk);
				if (has_a)
					load4(xa, ba, s + 4);
				run4(xb, bb);
				s += 4;
				if (!has_a)
					break;
			}
		}
		pa += static_cast<ptrdiff_t>(s - s0) * s8;
		pb += static_cast<ptrdiff_t>(s - s0) * s8;
		for (; s < s1; ++s) {
			const float x0 = __ldg(reinterpret_cast<const float *>(pa));
			const float x1 = __ldg(reinterpret_cast<const float *>(pb));
			const float x2 = __ldg(reinterpret_cast<const float *>(pa + khi));
			const float x3 = __ldg(reinterpret_cast<const float *>(pb + khi));
			float c[4] = { 0.f, 0.f, 0.f, 0.f };
			step3(c, x0, x1, x2, x3, __ldg(bf + s * 32));
			add4(d, c);
			pa += s8;
			pb += s8;
		}
	} else {
		// the block reaches past the last input: clamp (those taps are zero)
		const int kmax = src_dim - 1;
		const int kinc = PERM_K ? 1 : 4;
		for (int s = s0; s < s1; ++s) {
			const int k0 = min(kb + 8 * s + koff, kmax), k1 = min(kb + 8 * s + koff + kinc, kmax);
			const float x0 = __ldg(reinterpret_cast<const float *>(base_a + k0 * sk));
			const float x1 = __ldg(reinterpret_cast<const float *>(base_b + k0 * sk));
			const float x2 = __ldg(reinterpret_cast<const float *>(base_a + k1 * sk));
			const float x3 = __ldg(reinterpret_cast<const float *>(base_b + k1 * sk));
			float c[4] = { 0.f, 0.f, 0.f, 0.f };
			step3(c, x0, x1, x2, x3, __ldg(bf + s * 32));
			add4(d, c);
		}
	}
}

// D (m = gid / gid + 8, n = 2 tig, 2 tig + 1) -> outputs; mA, mB: the m that
// fragment rows gid and gid + 8 stand for.
__device__ __forceinline__ void store_group(const float (&d)[4], int g, int mA, int mB, int m_extent, int dst_dim,
                                            char *dst, ptrdiff_t dm, ptrdiff_t dko)
{
	const int tig = threadIdx.x & 3;
	const int o = g * 8 + 2 * tig;
	if (o < dst_dim) {
		if (mA < m_extent) *reinterpret_cast<float *>(dst + mA * dm + o * dko) = d[0];
		if (mB < m_extent) *reinterpret_cast<float *>(dst + mB * dm + o * dko) = d[2];
	}
	if (o + 1 < dst_dim) {
		if (mA < m_extent) *reinterpret_cast<float *>(dst + mA * dm + (o + 1) * dko) = d[1];
		if (mB < m_extent) *reinterpret_cast<float *>(dst + mB * dm + (o + 1) * dko) = d[3];
	}
}

// Output (o, m) is at dst + m * dm + o * dko. KSPLIT 1: a warp owns 16
// consecutive m and walks output groups [g0, g1). KSPLIT = kWideWarps (passes
// with few m, e.g. the horizontal pass after a strong vertical downscale): the
// CTA's warps share one 16-m tile and split each group's k-steps; the
// partial sums are added in warp order (deterministic) by warp 0.
// HORIZ: horizontal pass (m = rows, k = columns, B fragments with PERM_K).
// PAIR: 8-byte operand loads; the source plane's base and stride are
// multiples of 8 bytes, and in a vertical pass every tile of [tile_begin,
// tile_end) is whole, fragment rows gid and gid + 8 standing for the adjacent
// columns m0 + 2 gid and m0 + 2 gid + 1.
template <int KSPLIT, bool HORIZ, bool PAIR>
__global__ void __launch_bounds__(kWideWarps * 32)
wide_tc_kernel(WideTables w, int m_extent, int src_dim, int dst_dim, const char *__restrict__ src, ptrdiff_t sm,
               ptrdiff_t sk, char *__restrict__ dst, ptrdiff_t dm, ptrdiff_t dko, int groups_per_block, int tile_begin,
               int tile_end)
{
	__shared__ float4 red[KSPLIT > 1 ? KSPLIT * 32 : 1];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int gid = lane >> 2;
	const int tile = tile_begin + (KSPLIT > 1 ? blockIdx.x : blockIdx.x * kWideWarps + warp);
	if (tile >= tile_end)
		return;  // whole CTA when KSPLIT > 1
	const int m0 = tile * 16;
	const int mA = (!HORIZ && PAIR) ? m0 + 2 * gid : m0 + gid;
	const int mB = (!HORIZ && PAIR) ? m0 + 2 * gid + 1 : m0 + gid + 8;
	const int ma = min(mA, m_extent - 1), mb = min(mB, m_extent - 1);
	const int g0 = blockIdx.y * groups_per_block;
	const int g1 = min(w.groups, g0 + groups_per_block);
	const int KS = w.ksteps;
	const char *base_a = src + ma * sm, *base_b = src + mb * sm;

	for (int g = g0; g < g1; ++g) {
		float d[4] = { 0.f, 0.f, 0.f, 0.f };
		const int per = (KS + KSPLIT - 1) / KSPLIT;
		const int s0 = KSPLIT == 1 ? 0 : min(KS, warp * per), s1 = KSPLIT == 1 ? KS : min(KS, s0 + per);
		band_sum<HORIZ, PAIR>(d, w, g, s0, s1, src_dim, base_a, base_b, sk, src + m0 * sm, m_extent - m0, sm);
		if (KSPLIT == 1) {
			store_group(d, g, mA, mB, m_extent, dst_dim, dst, dm, dko);
		} else {
			red[warp * 32 + lane] = make_float4(d[0], d[1], d[2], d[3]);
			__syncthreads();
			if (warp == 0) {
				float t[4] = { 0.f, 0.f, 0.f, 0.f };
#pragma unroll
				for (int i = 0; i < KSPLIT; ++i) {
					const float4 v = red[i * 32 + lane];
					t[0] += v.x;
					t[1] += v.y;
					t[2] += v.z;
					t[3] += v.w;
				}
				store_group(t, g, mA, mB, m_extent, dst_dim, dst, dm, dko);
			}
			__syncthreads();
		}
	}
}

// Round an f32 to the nearest tf32 (ties away from zero), as cvt.rna.tf32.f32.
float tf32_round(float x)
{
	uint32_t u;
	std::memcpy(&u, &x, 4);
	if ((u & 0x7F800000u) != 0x7F800000u) {
		u += 0x1000u;
		u &= ~0x1FFFu;
	}
	float r;
	std::memcpy(&r, &u, 4);
	return r;
}

int sm_count()
{
	static int cached[64] = {};
	int dev = 0;
	cudaGetDevice(&dev);
	if (dev < 0 || dev >= 64)
		return 152;
	if (!cached[dev]) {
		int n = 0;
		cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
		cached[dev] = n > 0 ? n : 152;
	}
	return cached[dev];
}

uint32_t bits(float x)
{
	uint32_t u;
	std::memcpy(&u, &x, 4);
	return u;
}

} // namespace

void build_wide_tables(const float *f32, const unsigned *left, unsigned width, unsigned rows, bool perm_k,
                       std::vector<uint4> *frag, std::vector<int> *kbase, int *ksteps)
{
	const int groups = static_cast<int>((rows + 7) / 8);
	kbase->assign(groups, 0);
	int ks = 1;
	for (int g = 0; g < groups; ++g) {
		unsigned lo = ~0u, hi = 0;
		for (unsigned o = g * 8u; o < std::min(rows, g * 8u + 8); ++o) {
			lo = std::min(lo, left[o]);
			hi = std::max(hi, left[o] + width);
		}
		if (perm_k)
			lo &= ~1u;  // 8-byte aligned pairs of inputs
		(*kbase)[g] = static_cast<int>(lo);
		ks = std::max(ks, static_cast<int>((hi - lo + 7) / 8));
	}
	*ksteps = ks;
	frag->assign(static_cast<size_t>(groups) * ks * 32, uint4{ 0, 0, 0, 0 });
	auto tap = [&](unsigned o, long x) -> float {
		if (o >= rows)
			return 0.0f;
		const long k = x - static_cast<long>(left[o]);
		return (k >= 0 && k < static_cast<long>(width)) ? f32[static_cast<size_t>(o) * width + k] : 0.0f;
	};
	for (int g = 0; g < groups; ++g) {
		for (int s = 0; s < ks; ++s) {
			for (int lane = 0; lane < 32; ++lane) {
				const unsigned o = g * 8u + (lane >> 2);
				const int tig = lane & 3;
				// inputs of fragment k = tig and k = tig + 4 (see band_sum)
				const long x0 = (*kbase)[g] + 8L * s + (perm_k ? 2 * tig : tig);
				const long x1 = x0 + (perm_k ? 1 : 4);
				const float c0 = tap(o, x0), c1 = tap(o, x1);
				const float h0 = tf32_round(c0), h1 = tf32_round(c1);
				const float l0 = tf32_round(c0 - h0), l1 = tf32_round(c1 - h1);
				(*frag)[(static_cast<size_t>(g) * ks + s) * 32 + lane] = uint4{ bits(h0), bits(h1), bits(l0), bits(l1) };
			}
		}
	}
}

void build_umma_tables(const float *f32, const unsigned *left, unsigned width, unsigned rows,
                       std::vector<uint4> *chunks, std::vector<int> *chunk_begin, std::vector<int> *kbase)
{
	constexpr unsigned kOut = 64, kKC = 16;
	const unsigned tiles = (rows + kOut - 1) / kOut;
	chunk_begin->assign(tiles + 1, 0);
	kbase->assign(tiles, 0);
	int total = 0;
	for (unsigned t = 0; t < tiles; ++t) {
		unsigned lo = ~0u, hi = 0;
		for (unsigned o = t * kOut; o < std::min(rows, (t + 1) * kOut); ++o) {
			lo = std::min(lo, left[o]);
			hi = std::max(hi, left[o] + width);
		}
		(*kbase)[t] = static_cast<int>(lo);
		(*chunk_begin)[t] = total;
		total += static_cast<int>((hi - lo + kKC - 1) / kKC);
	}
	(*chunk_begin)[tiles] = total;
	// per chunk two 8-row blocks of 1024 words: row i < 64 holds the TF32
	// high part of output 64 t + i's taps, row 64 + i its remainder; element
	// (row, k) at (row / 8) * 128 + (k / 4) * 2048 + (row % 8) * 16 + (k % 4) * 4
	// bytes (K-major core matrices)
	chunks->assign(static_cast<size_t>(total) * 512, uint4{ 0, 0, 0, 0 });
	uint32_t *w32 = reinterpret_cast<uint32_t *>(chunks->data());
	for (unsigned t = 0; t < tiles; ++t) {
		const int nc = (*chunk_begin)[t + 1] - (*chunk_begin)[t];
		for (int c = 0; c < nc; ++c) {
			uint32_t *blk = w32 + static_cast<size_t>((*chunk_begin)[t] + c) * 2048;
			for (unsigned i = 0; i < kOut; ++i) {
				const unsigned o = t * kOut + i;
				if (o >= rows)
					continue;
				for (unsigned kk = 0; kk < kKC; ++kk) {
					const long x = (*kbase)[t] + static_cast<long>(kKC) * c + kk;
					const long k = x - static_cast<long>(left[o]);
					if (k < 0 || k >= static_cast<long>(width))
						continue;
					const float v = f32[static_cast<size_t>(o) * width + k];
					const float h = tf32_round(v);
					const unsigned step = kk / 8, k8 = kk % 8;
					auto at = [&](unsigned row) {
						return step * 1024 + ((row >> 3) * 128 + (k8 >> 2) * 2048 + (row & 7) * 16 + (k8 & 3) * 4) / 4;
					};
					blk[at(i)] = bits(h);
					blk[at(64 + i)] = bits(tf32_round(v - h));
				}
			}
		}
	}
}

namespace {

// Which form runs a vertical wide pass. ZG_WIDE_KERNEL=mma: the mma.sync
// form; =umma: the tcgen05 form wherever the plane and the band allow it;
// unset: the tcgen05 form when its tiles fill at least three quarters of the
// SMs (one tile is a long stream of products), else the mma.sync form. Bands
// wider than kUmmaMaxTaps stay on the mma.sync form: the tcgen05 form
// accumulates a whole band in tensor memory (2 products per 8 taps), and the
// tensor core's accumulation is not round-to-nearest.
constexpr int kUmmaMaxTaps = 160;

int wide_kernel_choice()
{
	const char *e = std::getenv("ZG_WIDE_KERNEL");
	if (e && std::strcmp(e, "mma") == 0)
		return 1;
	if (e && std::strcmp(e, "umma") == 0)
		return 2;
	return 0;
}

template <int KSPLIT, bool HORIZ, bool PAIR>
void launch_tiles(const PassLaunch &l, int m_extent, int src_dim, int dst_dim, ptrdiff_t sm, ptrdiff_t sk, ptrdiff_t dm,
                  ptrdiff_t dko, int gpb, int t0, int t1, cudaStream_t stream)
{
	if (t1 <= t0)
		return;
	const int bx = KSPLIT > 1 ? t1 - t0 : (t1 - t0 + kWideWarps - 1) / kWideWarps;
	const int by = (l.wide.groups + gpb - 1) / gpb;
	wide_tc_kernel<KSPLIT, HORIZ, PAIR><<<dim3(bx, by), kWideWarps * 32, 0, stream>>>(
		l.wide, m_extent, src_dim, dst_dim, static_cast<const char *>(l.src), sm, sk, static_cast<char *>(l.dst), dm, dko,
		gpb, t0, t1);
}

// One pass: aligned planes take 8-byte loads (in a vertical pass the whole
// 16-column tiles; a partial last tile runs in a second, 4-byte launch).
template <int KSPLIT>
void launch_pass_tiles(const PassLaunch &l, int m_extent, int src_dim, int dst_dim, ptrdiff_t sm, ptrdiff_t sk,
                       ptrdiff_t dm, ptrdiff_t dko, int gpb, bool aligned8, cudaStream_t stream)
{
	const int mtiles = (m_extent + 15) / 16;
	if (l.horizontal) {
		if (aligned8)
			launch_tiles<KSPLIT, true, true>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gpb, 0, mtiles, stream);
		else
			launch_tiles<KSPLIT, true, false>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gpb, 0, mtiles, stream);
		return;
	}
	const int whole = aligned8 ? m_extent / 16 : 0;
	launch_tiles<KSPLIT, false, true>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gpb, 0, whole, stream);
	launch_tiles<KSPLIT, false, false>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gpb, whole, mtiles, stream);
}

} // namespace

namespace {
thread_local int g_wide_forms = 0;
}

int wide_forms_used(bool reset)
{
	const int v = g_wide_forms;
	if (reset)
		g_wide_forms = 0;
	return v;
}

cudaError_t launch_wide(const PassLaunch &l, cudaStream_t stream)
{
	const int choice = wide_kernel_choice();
	if (l.wide.uchunk && !l.horizontal && choice != 1 && l.wide.umax_taps <= kUmmaMaxTaps &&
	    (choice == 2 || 4L * wide_umma_items(l) >= 3L * sm_count())) {
		const cudaError_t e = launch_wide_umma(l, stream);
		if (e != cudaErrorNotSupported) {
			g_wide_forms |= 2;
			return e;
		}
	}
	g_wide_forms |= 1;
	const int m_extent = static_cast<int>(l.lines);
	const int src_dim = static_cast<int>(l.t.input_width);
	const int dst_dim = static_cast<int>(l.t.rows);
	const ptrdiff_t sm = l.horizontal ? l.src_stride : 4, sk = l.horizontal ? 4 : l.src_stride;
	const ptrdiff_t dm = l.horizontal ? l.dst_stride : 4, dko = l.horizontal ? 4 : l.dst_stride;
	const int mtiles = (m_extent + 15) / 16;
	const bool aligned8 = reinterpret_cast<uintptr_t>(l.src) % 8 == 0 && l.src_stride % 8 == 0;
	const long sms = sm_count();
	const int gmin = (l.wide.groups + 65534) / 65535;  // grid y limit
	if (static_cast<long>(mtiles) * l.wide.groups < sms * 16 && l.wide.ksteps >= 2 * kWideWarps) {
		// few output tiles: split each group's k-steps across the CTA's warps
		launch_pass_tiles<kWideWarps>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gmin, aligned8, stream);
		return cudaGetLastError();
	}
	// enough warps for several waves on every SM, then longer runs of groups
	int gpb = static_cast<int>(std::max<long>(1, static_cast<long>(mtiles) * l.wide.groups / (sms * 64)));
	gpb = std::max(std::min(gpb, 8), gmin);
	launch_pass_tiles<1>(l, m_extent, src_dim, dst_dim, sm, sk, dm, dko, gpb, aligned8, stream);
	return cudaGetLastError();
}

} // namespace zg
