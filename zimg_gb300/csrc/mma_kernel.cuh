// Tensor-core variant of the fused streaming kernel for u16 samples (exact).
//
// Same streaming structure as fused_kernel.cuh (strips of 128 output columns,
// source lines through rings in shared memory), but both passes run as small
// banded matrix products on the tensor cores with mma.sync m16n8k16
// (fp16 operands, fp32 accumulation):
//
//   * samples are re-centred, v' = v - 2^(depth-1), exact in fp16 (the planner
//     only certifies depths up to 10, see below);
//   * each int16 tap is split c = hi + lo, hi = c - (c & 31) (a multiple of 32
//     with at most 11 significant bits), lo = c & 31, both exact in fp16;
//   * both halves multiply the same samples into one fp32 accumulator that
//     starts at 8192. The planner proved per output that
//     8192 + sum(|hi| + |lo|) * 2^(depth-1) < 2^24, so every product and every
//     partial sum is an integer representable in fp32: the accumulator holds
//     8192 + sum(c * v') exactly, and the rounding below reproduces zimg's
//     ((sum + 8192) >> 14) + 32768 with clamping (resize_impl.cpp:31-42).
//
// Fragment layouts follow the PTX ISA description of mma.m16n8k16 (.f16):
// groupID = lane >> 2, tig = lane & 3.
#pragma once

#include <cuda_fp16.h>

#include "fused.h"

namespace zg {
namespace mma_detail {

constexpr int kThreads = 256;             // 8 warps
constexpr int kWarps = kThreads / 32;
constexpr int kMidPitch = kStripW + 8;    // halfs per intermediate line (272 bytes)

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
	asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
	asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(p));
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(s));
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(p));
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(s));
}

// D += A * B, m16n8k16, f16 x f16 -> f32
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
	asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
	    "{%0, %1, %2, %3};\n"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc (exact 8192 + sum c*v') -> two packed, clamped zimg samples (low/high half).
// Both values in one paired fp32 multiply-add (round toward minus infinity,
// so floor((acc - 8192) / 2^14 + 1/2) lands in the low mantissa bits of
// 1.5*2^23 + offset), the low halves packed, and one s16x2 minimum with
// relu for the clamp to [0, pixel_max].
__device__ __forceinline__ uint32_t pack_u16x2(float acc0, float acc1, float magic, uint32_t pmax2)
{
	const float2 y = __ffma2_rd(make_float2(acc0, acc1), make_float2(6.103515625e-05f, 6.103515625e-05f),
	                            make_float2(magic, magic));
	// low 16 bits of y are the signed sample before clamping
	uint32_t q = __byte_perm(__float_as_uint(y.x), __float_as_uint(y.y), 0x5410);
	asm("min.relu.s16x2 %0, %0, %1;" : "+r"(q) : "r"(pmax2));
	return q;
}

// Two clamped samples (packed u16, each < 1024) -> centred fp16x2: the fp16
// with exponent 2^10 and mantissa q is exactly 1024 + q.
__device__ __forceinline__ uint32_t u16x2_to_centred_h2(uint32_t q, uint32_t bias_h2)
{
	const uint32_t v = q | 0x64006400u;
	const __half2 h = __hsub2(*reinterpret_cast<const __half2 *>(&v), *reinterpret_cast<const __half2 *>(&bias_h2));
	return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ int wrap(int s, int R)
{
	s = s >= R ? s - R : s;
	return s >= R ? s - R : s;
}

struct Item {
	const char *src;
	ptrdiff_t src_stride;
	char *dst;
	ptrdiff_t dst_stride;
	const uint4 *vfrag;
	const uint2 *hfrag;
	int src_w, src_h, dst_h, vec_ok;
	int c0, cols_valid, xlo, pxa, strip, sw;
	int g_begin, g_end, step_groups, depth;
	// this thread's place in line copies: chunk q0 of line offset l0, then
	// advance by (sl lines, sq chunks) per iteration
	int chunks, q0, l0, sl, sq;
	float magic;
	uint32_t pmax2, bias_h2;
};

__device__ __forceinline__ int find_job(const FusedJob *__restrict__ jobs, int num_jobs, int t)
{
	int lo = 0, hi = num_jobs - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (__ldg(&jobs[mid].item_begin) <= t)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ Item make_item(const FusedJob &J, int t)
{
	Item it;
	const int local = t - J.item_begin;
	const int seg = local / J.strips;
	it.strip = local - seg * J.strips;
	it.src = static_cast<const char *>(J.src);
	it.src_stride = J.src_stride;
	it.dst = static_cast<char *>(J.dst);
	it.dst_stride = J.dst_stride;
	it.vfrag = reinterpret_cast<const uint4 *>(J.v_dense);
	it.hfrag = reinterpret_cast<const uint2 *>(J.h_taps);
	it.src_w = J.src_w;
	it.src_h = J.src_h;
	it.dst_h = J.dst_h;
	it.vec_ok = J.vec_ok;
	it.sw = J.strip_w;
	it.c0 = it.strip * it.sw;
	it.cols_valid = min(it.sw, J.dst_w - it.c0);
	it.xlo = __ldg(J.win_col + 2 * it.strip);
	it.pxa = (__ldg(J.win_col + 2 * it.strip + 1) - it.xlo + 7) & ~7;
	it.g_begin = seg * J.seg_groups;
	it.g_end = min(J.groups, it.g_begin + J.seg_groups);
	it.step_groups = J.step_groups;
	it.depth = J.depth;
	it.magic = J.magic;
	const uint32_t pm = static_cast<uint32_t>(J.pixel_max);
	it.pmax2 = pm | (pm << 16);
	const __half2 b = __floats2half2_rn(1024.0f + J.offset, 1024.0f + J.offset);
	it.bias_h2 = *reinterpret_cast<const uint32_t *>(&b);
	it.chunks = it.pxa / 8;
	it.q0 = threadIdx.x % it.chunks;
	it.l0 = threadIdx.x / it.chunks;
	it.sl = kThreads / it.chunks;
	it.sq = kThreads % it.chunks;
	return it;
}

// Source lines [a, b) of the strip (raw u16) into staging slots; sa = a % SR.
__device__ __forceinline__ void load_lines(const Item &it, int a, int b, char *stage, int SR, int sa, int pitch)
{
	int y = a + it.l0, q = it.q0;
	for (; y < b; ) {
		const bool row_ok = y < it.src_h;
		const char *row = it.src + static_cast<ptrdiff_t>(row_ok ? y : 0) * it.src_stride;
		char *srow = stage + wrap(sa + (y - a), SR) * pitch * 2;
		const int gx = it.xlo + q * 8;
		if (it.vec_ok) {
			const int n = row_ok ? max(0, min(8, it.src_w - gx)) : 0;
			cp_async16(srow + q * 16, n ? row + static_cast<ptrdiff_t>(gx) * 2 : it.src, n * 2);
		} else {
			uint16_t *d = reinterpret_cast<uint16_t *>(srow + q * 16);
#pragma unroll
			for (int e = 0; e < 8; ++e)
				d[e] = (row_ok && gx + e < it.src_w) ? __ldg(reinterpret_cast<const uint16_t *>(row) + gx + e)
				                                      : static_cast<uint16_t>(0);
		}
		q += it.sq;
		y += it.sl;
		if (q >= it.chunks) {
			q -= it.chunks;
			++y;
		}
	}
}

// Raw staged lines this thread loaded -> centred fp16 lines (same mapping).
__device__ __forceinline__ void convert_lines(const Item &it, int a, int b, const char *stage, int SR, int sa,
                                              char *ring, int RR, int ra, int pitch)
{
	int y = a + it.l0, q = it.q0;
	for (; y < b; ) {
		const uint4 *s = reinterpret_cast<const uint4 *>(stage + wrap(sa + (y - a), SR) * pitch * 2);
		uint4 *d = reinterpret_cast<uint4 *>(ring + wrap(ra + (y - a), RR) * pitch * 2);
		uint4 u = s[q];
		u.x = u16x2_to_centred_h2(u.x, it.bias_h2);
		u.y = u16x2_to_centred_h2(u.y, it.bias_h2);
		u.z = u16x2_to_centred_h2(u.z, it.bias_h2);
		u.w = u16x2_to_centred_h2(u.w, it.bias_h2);
		d[q] = u;
		q += it.sq;
		y += it.sl;
		if (q >= it.chunks) {
			q -= it.chunks;
			++y;
		}
	}
}

// Vertical tap fragments of groups [g0, g1) into a shared slot.
template <int KV>
__device__ __forceinline__ void load_vfrag(const Item &it, int g0, int g1, char *slot)
{
	const char *src = reinterpret_cast<const char *>(it.vfrag) + static_cast<size_t>(g0) * KV * 2 * 32 * 16;
	const int n = (g1 - g0) * KV * 2 * 32;
	for (int i = threadIdx.x; i < n; i += kThreads)
		cp_async16(slot + i * 16, src + i * 16, 16);
}

// Horizontal pass on 16-line blocks: for each column group cg (8 outputs),
// D[16 lines][8] = sum over KH*16 columns starting at hbase[cg] - xlo.
// A: lines of `in` (ring of IR lines, line a in slot ia; ldmatrix with a row
// address per line), B: tap fragments from shared memory.
// out: TO_RING: centred fp16 into ring slots (line a in slot oa of OR);
//      else: packed u16 into the staged output tile (line a -> tile row 0).
template <int KH, bool TO_RING>
__device__ __forceinline__ void h_pass(const Item &it, const int *hbase, const uint2 *hfrag, const char *in, int IR,
                                       int ia, int in_pitch, int a, int b, char *out, int OR, int oa, int out_pitch)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int gid = lane >> 2, tig = lane & 3;
	const int ncg = (it.cols_valid + 7) / 8;
	for (int cg = warp; cg < ncg; cg += kWarps) {
		uint2 bf[KH][2];
#pragma unroll
		for (int ks = 0; ks < KH; ++ks)
#pragma unroll
			for (int h = 0; h < 2; ++h)
				bf[ks][h] = hfrag[((cg * KH + ks) * 2 + h) * 32 + lane];
		const int col0 = hbase[cg] - it.xlo;
		for (int y0 = a; y0 < b; y0 += 16) {
			// row address for this lane: line y0 + (lane & 15), column block (lane >> 4) * 8
			const char *rowp = in + wrap(ia + (y0 - a) + (lane & 15), IR) * in_pitch * 2 + (col0 + (lane >> 4) * 8) * 2;
			float d[4] = { 8192.0f, 8192.0f, 8192.0f, 8192.0f };
#pragma unroll
			for (int ks = 0; ks < KH; ++ks) {
				uint32_t af[4];
				// ldmatrix gives matrices (rows 0-7, cols 0-7), (rows 8-15, cols 0-7),
				// (rows 0-7, cols 8-15), (rows 8-15, cols 8-15): a0..a3 order
				ldsm_x4(af[0], af[1], af[2], af[3], rowp + ks * 32);
				mma16816(d, af, bf[ks][0].x, bf[ks][0].y);
				mma16816(d, af, bf[ks][1].x, bf[ks][1].y);
			}
			const uint32_t q01 = pack_u16x2(d[0], d[1], it.magic, it.pmax2);  // line y0+gid, cols 2tig..
			const uint32_t q23 = pack_u16x2(d[2], d[3], it.magic, it.pmax2);  // line y0+gid+8
			const int col = cg * 8 + 2 * tig;
			if (TO_RING) {
				const int sa = wrap(oa + (y0 - a) + gid, OR), sb = wrap(oa + (y0 - a) + gid + 8, OR);
				*reinterpret_cast<uint32_t *>(out + sa * out_pitch * 2 + col * 2) = u16x2_to_centred_h2(q01, it.bias_h2);
				*reinterpret_cast<uint32_t *>(out + sb * out_pitch * 2 + col * 2) = u16x2_to_centred_h2(q23, it.bias_h2);
			} else {
				*reinterpret_cast<uint32_t *>(out + (y0 - a + gid) * out_pitch * 2 + col * 2) = q01;
				*reinterpret_cast<uint32_t *>(out + (y0 - a + gid + 8) * out_pitch * 2 + col * 2) = q23;
			}
		}
	}
}

// Vertical pass for one 16-row group: D[16 rows][8 cols] = sum over KV*16
// lines from vbase of taps * in[line][col]. A: tap fragments (shared slot),
// B: lines of `in` (ring of IR lines, line vbase in slot iv; ldmatrix.trans).
// Warps [wfirst, wfirst + wcount) take columns [0, ncols) 16 at a time.
// TO_CENTRED: centred fp16 rows (tile of 16 lines); else packed u16 rows.
template <int KV, bool TO_CENTRED>
__device__ __forceinline__ void v_pass(const Item &it, const uint4 *afrag, const char *in, int IR, int iv,
                                       int in_pitch, int ncols, int wfirst, int wcount, char *out, int out_pitch)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int wi = warp - wfirst;
	if (wi < 0 || wi >= wcount)
		return;
	const int gid = lane >> 2, tig = lane & 3;
	uint4 af[KV][2];
#pragma unroll
	for (int ks = 0; ks < KV; ++ks)
#pragma unroll
		for (int h = 0; h < 2; ++h)
			af[ks][h] = afrag[(ks * 2 + h) * 32 + lane];
	// lane's ldmatrix row: line vbase + ks*16 + (lane & 7) + ((lane >> 3) & 1) * 8, column +(lane >> 4) * 8
	const int krow = (lane & 7) + ((lane >> 3) & 1) * 8;
	const int coff = (lane >> 4) * 8;
	const char *rowp[KV];
#pragma unroll
	for (int ks = 0; ks < KV; ++ks)
		rowp[ks] = in + wrap(iv + ks * 16 + krow, IR) * in_pitch * 2 + coff * 2;
	for (int x0 = wi * 16; x0 < ncols; x0 += wcount * 16) {
		float d0[4] = { 8192.0f, 8192.0f, 8192.0f, 8192.0f };
		float d1[4] = { 8192.0f, 8192.0f, 8192.0f, 8192.0f };
#pragma unroll
		for (int ks = 0; ks < KV; ++ks) {
			uint32_t b0, b1, b2, b3;
			ldsm_x4_trans(b0, b1, b2, b3, rowp[ks] + x0 * 2);
			const uint32_t ahi[4] = { af[ks][0].x, af[ks][0].y, af[ks][0].z, af[ks][0].w };
			const uint32_t alo[4] = { af[ks][1].x, af[ks][1].y, af[ks][1].z, af[ks][1].w };
			mma16816(d0, ahi, b0, b1);
			mma16816(d0, alo, b0, b1);
			mma16816(d1, ahi, b2, b3);
			mma16816(d1, alo, b2, b3);
		}
#pragma unroll
		for (int nb = 0; nb < 2; ++nb) {
			const float *d = nb ? d1 : d0;
			uint32_t q01 = pack_u16x2(d[0], d[1], it.magic, it.pmax2);  // row gid
			uint32_t q23 = pack_u16x2(d[2], d[3], it.magic, it.pmax2);  // row gid + 8
			if (TO_CENTRED) {
				q01 = u16x2_to_centred_h2(q01, it.bias_h2);
				q23 = u16x2_to_centred_h2(q23, it.bias_h2);
			}
			const int col = x0 + nb * 8 + 2 * tig;
			*reinterpret_cast<uint32_t *>(out + gid * out_pitch * 2 + col * 2) = q01;
			*reinterpret_cast<uint32_t *>(out + (gid + 8) * out_pitch * 2 + col * 2) = q23;
		}
	}
}

// Staged output tile (rows [0, nrows) of packed u16, out_pitch halfs) ->
// destination rows r0.., strip columns, 16-byte stores where whole.
__device__ __forceinline__ void store_tile(const Item &it, const char *tile, int out_pitch, int r0, int nrows)
{
	const int shift = it.sw == 128 ? 4 : 3;  // chunks of 8 columns per row: 16 or 8
	const int rows = min(nrows, it.dst_h - r0);
	for (int i = threadIdx.x; i < (rows << shift); i += kThreads) {
		const int r = i >> shift, q = i & ((1 << shift) - 1);
		const int col = q * 8;
		if (col >= it.cols_valid)
			continue;
		const uint4 v = *reinterpret_cast<const uint4 *>(tile + r * out_pitch * 2 + col * 2);
		uint16_t *d = reinterpret_cast<uint16_t *>(it.dst + static_cast<ptrdiff_t>(r0 + r) * it.dst_stride) + it.c0 + col;
		if (it.vec_ok && col + 8 <= it.cols_valid) {
			*reinterpret_cast<uint4 *>(d) = v;
		} else {
			const uint32_t w[4] = { v.x, v.y, v.z, v.w };
			for (int e = 0; e < 8 && col + e < it.cols_valid; ++e)
				d[e] = static_cast<uint16_t>(w[e >> 1] >> (16 * (e & 1)));
		}
	}
}

__device__ __forceinline__ void wait_groups(int pending)
{
	// cp.async.wait_group takes an immediate
	switch (pending) {
	case 0: cp_async_wait<0>(); break;
	case 1: cp_async_wait<1>(); break;
	case 2: cp_async_wait<2>(); break;
	case 3: cp_async_wait<3>(); break;
	default: cp_async_wait<4>(); break;
	}
}

// Kernel. Shared memory (SmemLayout): staging ring of raw u16 lines, ring of
// fp16 source lines, ring of fp16 intermediate lines (H-first) or 16 fp16
// intermediate lines (V-first), the staged output tile, the strip's
// horizontal tap fragments, depth+1 slots of vertical tap fragments,
// column-group bases and group bases. Lines of step k + depth are in flight
// while step k computes.
template <bool H_FIRST, int KV, int KH>
__global__ void __launch_bounds__(kThreads, 3)
mma_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_items, const __grid_constant__ FusedJob single,
           const __grid_constant__ SmemLayout L)
{
	extern __shared__ float4 smem4[];
	char *smem = reinterpret_cast<char *>(smem4);
	char *stage = smem + L.stage_off;
	char *src_ring = smem + L.in_off;     // fp16 source lines
	char *mid = smem + L.ring_off;        // H-first: fp16 intermediate lines
	char *I = smem + L.i_off;             // V-first: 16 fp16 intermediate lines; then the output tile
	char *tile = smem + L.tile_off;       // staged output rows (packed u16)
	const uint2 *hfrag = reinterpret_cast<const uint2 *>(smem + L.htaps_off);
	char *vslots = smem + L.vcoef_off;
	int *vb = reinterpret_cast<int *>(smem + L.vbase_off);
	int *hb = reinterpret_cast<int *>(smem + L.hleft_off);
	const int SR = L.stage_rows, IR = L.in_rows, MR = L.ring_rows;
	const int slot_bytes = L.step_groups * KV * 2 * 32 * 16;
	const int tile_pitch = L.tile_pitch;

	// Lines a pass reads past the last loaded one hold finite values.
	for (int i = threadIdx.x; i < L.htaps_off / 16; i += kThreads)
		smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
	__syncthreads();

	for (int t = blockIdx.x; t < total_items; t += gridDim.x) {
		const FusedJob *Jp = jobs ? &jobs[find_job(jobs, num_jobs, t)] : &single;
		const Item it = make_item(*Jp, t);
		for (int g = it.g_begin + threadIdx.x; g < it.g_end; g += kThreads)
			vb[g - it.g_begin] = __ldg(Jp->v_base + g);
		const int cgroups = (Jp->dst_w + 7) / 8;
		for (int i = threadIdx.x; i < it.sw / 8; i += kThreads)
			hb[i] = __ldg(Jp->h_left + min(it.c0 / 8 + i, cgroups - 1));
		{
			// the strip's horizontal tap fragments (one per column group)
			const int ncg = min(it.sw / 8, cgroups - it.c0 / 8);
			const char *src = reinterpret_cast<const char *>(it.hfrag) + static_cast<size_t>(it.c0 / 8) * KH * 2 * 32 * 8;
			for (int i = threadIdx.x; i < ncg * KH * 2 * 32 * 8 / 16; i += kThreads)
				cp_async16(smem + L.htaps_off + i * 16, src + i * 16, 16);
		}
		__syncthreads();

		const int nsteps = (it.g_end - it.g_begin + it.step_groups - 1) / it.step_groups;
		const int D = it.depth;
		auto groups_of = [&](int k, int *g0, int *g1) {
			*g0 = it.g_begin + k * it.step_groups;
			*g1 = min(it.g_end, *g0 + it.step_groups);
		};
		auto hi_of = [&](int k) {
			int g0, g1;
			groups_of(k, &g0, &g1);
			return vb[g1 - 1 - it.g_begin] + KV * 16;
		};
		// prologue: steps 0 .. D-1 in flight, one commit group each
		int issued_hi = vb[0];
		for (int k = 0; k < D; ++k) {
			if (k < nsteps) {
				int g0, g1;
				groups_of(k, &g0, &g1);
				const int hi = hi_of(k);
				load_lines(it, issued_hi, hi, stage, SR, issued_hi % SR, L.pitch);
				load_vfrag<KV>(it, g0, g1, vslots + (k % (D + 1)) * slot_bytes);
				issued_hi = hi;
			}
			cp_async_commit();
		}
		__syncthreads();  // lines stored by plain loads (unaligned planes) are visible to every converter

		int lo_cur = vb[0];
		for (int k = 0; k < nsteps; ++k) {
			int g0, g1;
			groups_of(k, &g0, &g1);
			const int hi_cur = hi_of(k);
			if (k + D < nsteps) {
				int n0, n1;
				groups_of(k + D, &n0, &n1);
				const int hi = hi_of(k + D);
				load_lines(it, issued_hi, hi, stage, SR, issued_hi % SR, L.pitch);
				load_vfrag<KV>(it, n0, n1, vslots + ((k + D) % (D + 1)) * slot_bytes);
				issued_hi = hi;
			}
			cp_async_commit();
			wait_groups(D);
			convert_lines(it, lo_cur, hi_cur, stage, SR, lo_cur % SR, src_ring, IR, lo_cur % IR, L.pitch);
			__syncthreads();
			const uint4 *afrag = reinterpret_cast<const uint4 *>(vslots + (k % (D + 1)) * slot_bytes);
			if (H_FIRST) {
				h_pass<KH, true>(it, hb, hfrag, src_ring, IR, lo_cur % IR, L.pitch, lo_cur, hi_cur, mid, MR,
				                 lo_cur % MR, kMidPitch);
				__syncthreads();
				const int ng = g1 - g0;
				const int wpg = kWarps / ng;  // ng <= step_groups <= kWarps / 2
				const int gi = (threadIdx.x >> 5) / wpg;
				if (gi < ng) {
					const int vbase = vb[g0 + gi - it.g_begin];
					v_pass<KV, false>(it, afrag + gi * KV * 2 * 32, mid, MR, vbase % MR, kMidPitch,
					                  (it.cols_valid + 15) & ~15, gi * wpg, wpg, tile + gi * 16 * tile_pitch * 2,
					                  tile_pitch);
				}
				__syncthreads();
				store_tile(it, tile, tile_pitch, g0 * 16, ng * 16);
			} else {
				// one 16-row group per step: ring -> I (16 lines x pxa) -> tile -> destination
				const int vbase = vb[g0 - it.g_begin];
				v_pass<KV, true>(it, afrag, src_ring, IR, vbase % IR, L.pitch, it.pxa, 0, kWarps, I, L.pitch);
				__syncthreads();
				h_pass<KH, false>(it, hb, hfrag, I, 1 << 30, 0, L.pitch, 0, 16, tile, 1, 0, tile_pitch);
				__syncthreads();
				store_tile(it, tile, tile_pitch, g0 * 16, 16);
			}
			__syncthreads();  // slots of step k are reused by step k + D + 1; the tile by step k + 1
			lo_cur = hi_cur;
		}
		cp_async_wait<0>();
		__syncthreads();
	}
}

} // namespace mma_detail
} // namespace zg
