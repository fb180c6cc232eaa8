// The fused two-pass streaming kernel (template). Instantiated per variant in
// fused_inst_*.cu.
//
// A work item is one strip of 128 output columns over one segment of output
// rows. The CTA walks the segment in steps of step_groups * 4 output rows.
// Source lines enter a ring of lines in shared memory by cp.async one step
// ahead of use, as zimg's graph keeps a ring of lines per filter
// (zimg.h:387-396), so each source line is read from HBM once per strip.
//
//   V-first step:  ring (source lines) --V--> I (intermediate lines of the
//                  step) --H--> destination rows
//   H-first step:  new source lines --H--> ring (intermediate lines)
//                  ring --V--> destination rows
//
// u16 samples are staged raw and converted once to exact centred floats, or
// (INT, depths the float proof cannot cover) to centred int32 values held as
// float bits, summed in zimg's int32 arithmetic. The grid is persistent: in a
// batch CTAs take guided chunks of the units (work_chunks.cuh), otherwise an
// equal contiguous share each.
#pragma once

#include "fused.h"
#include "work_chunks.cuh"

namespace zg {
namespace fused_detail {

constexpr int kThreads = kStreamThreads;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, int src_bytes)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
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

// u16 exact arithmetic: acc holds 8192 + sum(tap * (v - offset)) as an exact
// integer; round down acc / 2^14 onto the integer grid of [2^23, 2^24) and
// clamp there. The low 16 bits of the result are zimg's packed sample
// ((sum + 8192) >> 14, clamped, resize_impl.cpp:36-42).
__device__ __forceinline__ float u16_round(float acc, float magic, float pixel_max)
{
	float y = __fmaf_rd(acc, 6.103515625e-05f, magic);
	return fminf(fmaxf(y, 12582912.0f), 12582912.0f + pixel_max);
}

// zimg's int32 rounding (pack_pixel_u16, resize_impl.cpp:36-42): acc holds
// 8192 + sum(tap * (v - 32768)); (acc >> 14) + 32768 clamped to [0, pixel_max].
__device__ __forceinline__ int u16_round_int(int acc, int pixel_max)
{
	return min(max((acc >> 14) + 32768, 0), pixel_max);
}

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

// Registers-resident description of one work item.
struct Item {
	const char *src;
	ptrdiff_t src_stride;
	char *dst;
	ptrdiff_t dst_stride;
	const char *v_dense;
	const int *v_base;
	int src_w, src_h, dst_h, vec_ok;
	int c0, cols_valid, xlo, pxa;
	int g_begin, g_end, step_groups, units;
	float magic, pixel_max, offset;
};

// Units t .. t_end - 1 of job J that lie in the strip of unit t, at most
// L.seg_groups groups of them: a work item. A job's units are its (strip,
// streaming step) pairs, strip-major.
template <int HW>
__device__ __forceinline__ Item make_item(const FusedJob &J, int t, int t_end, char *smem, const SmemLayout &L)
{
	Item it;
	const int local = t - J.item_begin;
	const int strip = local / J.segments;
	const int step0 = local - strip * J.segments;
	it.units = max(1, min(min(J.segments - step0, t_end - t), L.seg_groups / J.step_groups));
	it.src = static_cast<const char *>(J.src);
	it.src_stride = J.src_stride;
	it.dst = static_cast<char *>(J.dst);
	it.dst_stride = J.dst_stride;
	it.v_dense = reinterpret_cast<const char *>(J.v_dense);
	it.v_base = J.v_base;
	it.src_w = J.src_w;
	it.src_h = J.src_h;
	it.dst_h = J.dst_h;
	it.vec_ok = J.vec_ok;
	it.c0 = strip * kStripW;
	it.cols_valid = min(kStripW, J.dst_w - it.c0);
	it.xlo = __ldg(J.win_col + 2 * strip);
	it.pxa = (__ldg(J.win_col + 2 * strip + 1) - it.xlo + 7) & ~7;
	it.g_begin = step0 * J.step_groups;
	it.g_end = min(J.groups, (step0 + it.units) * J.step_groups);
	it.step_groups = J.step_groups;
	it.magic = J.magic;
	it.pixel_max = J.pixel_max;
	it.offset = J.offset;

	// per-item tables: h taps and left offsets of the strip, group bases
	const char *ht = reinterpret_cast<const char *>(J.h_taps) + static_cast<size_t>(it.c0) * HW * 4;
	const int tap_bytes = it.cols_valid * HW * 4;
	for (int i = threadIdx.x; i < kStripW * HW / 4; i += kThreads) {
		const int n = max(0, min(16, tap_bytes - i * 16));
		cp_async16(smem + L.htaps_off + i * 16, n ? ht + i * 16 : ht, n);
	}
	for (int i = threadIdx.x; i < kStripW / 4; i += kThreads) {
		const int n = max(0, min(4, it.cols_valid - 4 * i));
		cp_async16(smem + L.hleft_off + i * 16, n ? J.h_left + it.c0 + 4 * i : J.h_left, n * 4);
	}
	int *vb = reinterpret_cast<int *>(smem + L.vbase_off);
	for (int g = it.g_begin + threadIdx.x; g < it.g_end; g += kThreads)
		vb[g - it.g_begin] = __ldg(J.v_base + g);
	return it;
}

// Lines [a, b) of the source strip into ring slots (line & mask) of `ring`
// (pitch elements of E bytes per line), zero outside the plane. Aligned
// planes: thread t copies 16-byte chunk t % chunks of lines a + t / chunks,
// then every kThreads / chunks lines further (one address step per line).
// Otherwise warp w takes lines a + w, a + w + 4, ... sample by sample.
template <bool U16>
__device__ __forceinline__ void load_lines(const Item &it, int a, int b, char *ring, int mask, int pitch)
{
	constexpr int E = U16 ? 2 : 4;
	constexpr int PER = 16 / E;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if (it.vec_ok) {
		const int chunks = it.pxa / PER;
		const int lpp = kThreads / chunks;
		if (lpp == 0) {
			// strips wider than kThreads chunks: warp per line
			for (int y = a + warp; y < b; y += kWarps) {
				const bool row_ok = y < it.src_h;
				const char *row = it.src + static_cast<ptrdiff_t>(row_ok ? y : 0) * it.src_stride;
				char *srow = ring + (y & mask) * pitch * E;
				for (int q = lane; q < chunks; q += 32) {
					const int gx = it.xlo + q * PER;
					const int n = row_ok ? max(0, min(PER, it.src_w - gx)) : 0;
					cp_async16(srow + q * 16, n ? row + static_cast<ptrdiff_t>(gx) * E : it.src, n * E);
				}
			}
			return;
		}
		const int q = threadIdx.x % chunks, l0 = threadIdx.x / chunks;
		if (l0 >= lpp)
			return;
		const int gx = it.xlo + q * PER;
		const int nb = max(0, min(PER, it.src_w - gx)) * E;
		const char *src = it.src + (nb ? static_cast<ptrdiff_t>(gx) * E : 0) + static_cast<ptrdiff_t>(a + l0) * it.src_stride;
		const ptrdiff_t step = static_cast<ptrdiff_t>(lpp) * it.src_stride;
		for (int y = a + l0; y < b; y += lpp, src += step) {
			const bool ok = y < it.src_h && nb;
			cp_async16(ring + ((y & mask) * pitch * E) + q * 16, ok ? src : it.src, ok ? nb : 0);
		}
		return;
	}
	for (int y = a + warp; y < b; y += kWarps) {
		const bool row_ok = y < it.src_h;
		const char *row = it.src + static_cast<ptrdiff_t>(row_ok ? y : 0) * it.src_stride;
		char *srow = ring + (y & mask) * pitch * E;
		if (!U16) {
			for (int x = lane; x < it.pxa; x += 32) {
				const int gx = it.xlo + x;
				const bool ok = row_ok && gx < it.src_w;
				cp_async4(srow + x * 4, ok ? row + static_cast<ptrdiff_t>(gx) * 4 : it.src, ok ? 4 : 0);
			}
		} else {
			for (int x = lane; x < it.pxa; x += 32) {
				const int gx = it.xlo + x;
				const bool ok = row_ok && gx < it.src_w;
				reinterpret_cast<uint16_t *>(srow)[x] =
					ok ? __ldg(reinterpret_cast<const uint16_t *>(row) + gx) : static_cast<uint16_t>(0);
			}
		}
	}
}

// Convert the u16 lines this thread loaded with load_lines(a, b) from the
// raw staging ring to centred floats in `ring` (INT: v - 32768 as int32 bits).
template <bool INT>
__device__ __forceinline__ void convert_chunk(const char *srow, float *drow, int q, float bias)
{
	const uint4 u = *reinterpret_cast<const uint4 *>(srow + q * 16);
	const uint32_t w[4] = { u.x, u.y, u.z, u.w };
	float f[8];
#pragma unroll
	for (int k = 0; k < 8; ++k) {
		const uint32_t v = (w[k >> 1] >> (16 * (k & 1))) & 0xFFFFu;
		f[k] = INT ? __int_as_float(static_cast<int>(v) - 32768) : __int_as_float(0x4B000000 | v) - bias;
	}
	*reinterpret_cast<float4 *>(drow + q * 8) = make_float4(f[0], f[1], f[2], f[3]);
	*reinterpret_cast<float4 *>(drow + q * 8 + 4) = make_float4(f[4], f[5], f[6], f[7]);
}

// Convert the u16 lines [a, b) from the raw staging ring to centred floats
// in `ring`. With cp.async copies each thread converts exactly the chunks it
// copied (the mapping of load_lines); plain loads were made visible by a
// CTA barrier, so any mapping serves.
template <bool INT>
__device__ __forceinline__ void convert_lines(const Item &it, int a, int b, const char *stage, int smask,
                                              float *ring, int rmask, int pitch)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const float bias = 8388608.0f + it.offset;
	const int chunks = it.pxa / 8;
	const int lpp = kThreads / chunks;
	if (it.vec_ok && lpp) {
		const int q = threadIdx.x % chunks, l0 = threadIdx.x / chunks;
		if (l0 >= lpp)
			return;
		for (int y = a + l0; y < b; y += lpp)
			convert_chunk<INT>(stage + (y & smask) * pitch * 2, ring + (y & rmask) * pitch, q, bias);
		return;
	}
	for (int y = a + warp; y < b; y += kWarps) {
		const char *srow = stage + (y & smask) * pitch * 2;
		float *drow = ring + (y & rmask) * pitch;
		for (int q = lane; q < chunks; q += 32)
			convert_chunk<INT>(srow, drow, q, bias);
	}
}

// Horizontal pass over lines [a, b): out[y][c] = sum_k taps[c][k] * in[y][left[c] - xlo + k].
// Thread = output column; two lines per iteration for independent chains.
// FINAL: write destination rows (row index = r0 + (y - a)); else write ring
// slots (y & omask) of `out`.
template <bool U16, bool FINAL, int HW, bool INT = false>
__device__ __forceinline__ void h_pass(const Item &it, const char *smem, const SmemLayout &L, const float *in,
                                       int imask, int a, int b, float *out, int omask, int r0)
{
	const int c = threadIdx.x;
	const bool col_ok = c < it.cols_valid;
	float taps[HW];
	const float2 *tp = reinterpret_cast<const float2 *>(smem + L.htaps_off) + c * (HW / 2);
#pragma unroll
	for (int k = 0; k < HW / 2; ++k) {
		const float2 t2 = tp[k];
		taps[2 * k] = t2.x;
		taps[2 * k + 1] = t2.y;
	}
	const int l = col_ok ? reinterpret_cast<const int *>(smem + L.hleft_off)[c] - it.xlo : 0;
	const float init = U16 ? 8192.0f : 0.0f;
	const int pitch = L.pitch;
	if constexpr (INT) {
		// zimg's int32 sums (taps and centred samples as int32 bits)
		const int pmax = static_cast<int>(it.pixel_max);
		for (int y = a; y < b; y += 2) {
			const bool two = y + 1 < b;
			const float *r0p = in + (y & imask) * pitch + l;
			const float *r1p = in + ((y + 1) & imask) * pitch + l;
			int acc0 = 8192, acc1 = 8192;
#pragma unroll
			for (int k = 0; k < HW; ++k) {
				const int t = __float_as_int(taps[k]);
				acc0 += t * __float_as_int(r0p[k]);
				acc1 += t * __float_as_int(r1p[k]);
			}
			const int q0 = u16_round_int(acc0, pmax), q1 = u16_round_int(acc1, pmax);
			if (!FINAL) {
				out[(y & omask) * kStripW + c] = __int_as_float(q0 - 32768);
				if (two)
					out[((y + 1) & omask) * kStripW + c] = __int_as_float(q1 - 32768);
			} else if (col_ok) {
				const int oy = r0 + (y - a);
				char *d0 = it.dst + static_cast<ptrdiff_t>(oy) * it.dst_stride;
				if (oy < it.dst_h)
					reinterpret_cast<uint16_t *>(d0)[it.c0 + c] = static_cast<uint16_t>(q0);
				if (two && oy + 1 < it.dst_h)
					reinterpret_cast<uint16_t *>(d0 + it.dst_stride)[it.c0 + c] = static_cast<uint16_t>(q1);
			}
		}
		return;
	}
	for (int y = a; y < b; y += 2) {
		const bool two = y + 1 < b;
		const float *r0p = in + (y & imask) * pitch + l;
		const float *r1p = in + ((y + 1) & imask) * pitch + l;
		// the two lines in one paired FMA per tap (two independent
		// round-to-nearest FMAs, as the scalar form)
		float2 acc = make_float2(init, init);
#pragma unroll
		for (int k = 0; k < HW; ++k)
			acc = __ffma2_rn(make_float2(taps[k], taps[k]), make_float2(r0p[k], r1p[k]), acc);
		const float acc0 = acc.x, acc1 = acc.y;
		if (!FINAL) {
			float v0 = acc0, v1 = acc1;
			if (U16) {
				v0 = u16_round(acc0, it.magic, it.pixel_max) - it.magic;
				v1 = u16_round(acc1, it.magic, it.pixel_max) - it.magic;
			}
			out[(y & omask) * kStripW + c] = v0;
			if (two)
				out[((y + 1) & omask) * kStripW + c] = v1;
		} else if (col_ok) {
			const int oy = r0 + (y - a);
			char *d0 = it.dst + static_cast<ptrdiff_t>(oy) * it.dst_stride;
			if (U16) {
				const uint32_t q0 = __float_as_uint(u16_round(acc0, it.magic, it.pixel_max)) & 0xFFFFu;
				const uint32_t q1 = __float_as_uint(u16_round(acc1, it.magic, it.pixel_max)) & 0xFFFFu;
				if (oy < it.dst_h)
					reinterpret_cast<uint16_t *>(d0)[it.c0 + c] = static_cast<uint16_t>(q0);
				if (two && oy + 1 < it.dst_h)
					reinterpret_cast<uint16_t *>(d0 + it.dst_stride)[it.c0 + c] = static_cast<uint16_t>(q1);
			} else {
				if (oy < it.dst_h)
					reinterpret_cast<float *>(d0)[it.c0 + c] = acc0;
				if (two && oy + 1 < it.dst_h)
					reinterpret_cast<float *>(d0 + it.dst_stride)[it.c0 + c] = acc1;
			}
		}
	}
}

// Vertical pass for groups [g0, g1): out line (g - g0)*4 + j, columns 4q..4q+3:
//   sum_s dense[g][s][j] * in[(base[g] + s) & imask][4q + e]
// FINAL: destination rows g*4 + j (columns c0 + 4q ...); else lines of I.
template <bool U16, bool FINAL, int VS, int kGroup, bool INT = false>
__device__ __forceinline__ void v_pass(const Item &it, const char *smem, const SmemLayout &L, const float *in,
                                       int imask, int in_pitch, int g0, int g1, const float *coef, int quads,
                                       float *I, int i_pitch)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const float init = U16 ? 8192.0f : 0.0f;
	const int ng = g1 - g0;
	const int wpg = ng >= kWarps ? 1 : kWarps / ng;  // warps per group
	const int *vb = reinterpret_cast<const int *>(smem + L.vbase_off);
	for (int gi = warp / wpg; gi < ng; gi += kWarps / wpg) {
		const int g = g0 + gi;
		const int base = vb[g - it.g_begin];
		const float *cf = coef + gi * VS * kGroup;  // [line][row] taps of the group's rows
		int off[VS];
#pragma unroll
		for (int s = 0; s < VS; ++s)
			off[s] = ((base + s) & imask) * in_pitch;
		for (int q = (warp % wpg) * 32 + lane; q < quads; q += wpg * 32) {
			if constexpr (INT) {
				// zimg's int32 sums (taps and centred samples as int32 bits)
				int acc[kGroup][4];
#pragma unroll
				for (int j = 0; j < kGroup; ++j)
					acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 8192;
#pragma unroll
				for (int s = 0; s < VS; ++s) {
					const int4 x = *reinterpret_cast<const int4 *>(in + off[s] + 4 * q);
#pragma unroll
					for (int j = 0; j < kGroup; ++j) {
						const int cj = __float_as_int(cf[s * kGroup + j]);
						acc[j][0] += cj * x.x;
						acc[j][1] += cj * x.y;
						acc[j][2] += cj * x.z;
						acc[j][3] += cj * x.w;
					}
				}
				const int pmax = static_cast<int>(it.pixel_max);
#pragma unroll
				for (int j = 0; j < kGroup; ++j) {
					int u[4];
#pragma unroll
					for (int e = 0; e < 4; ++e)
						u[e] = u16_round_int(acc[j][e], pmax);
					if (!FINAL) {
						*reinterpret_cast<int4 *>(I + (gi * kGroup + j) * i_pitch + 4 * q) =
							make_int4(u[0] - 32768, u[1] - 32768, u[2] - 32768, u[3] - 32768);
					} else {
						const int r = g * kGroup + j;
						if (r >= it.dst_h)
							continue;
						const int x0 = 4 * q;
						uint16_t *d = reinterpret_cast<uint16_t *>(it.dst + static_cast<ptrdiff_t>(r) * it.dst_stride) +
						              it.c0 + x0;
						if (it.vec_ok && x0 + 3 < it.cols_valid) {
							*reinterpret_cast<uint2 *>(d) = make_uint2(static_cast<uint32_t>(u[0]) | (static_cast<uint32_t>(u[1]) << 16),
							                                           static_cast<uint32_t>(u[2]) | (static_cast<uint32_t>(u[3]) << 16));
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < it.cols_valid)
									d[e] = static_cast<uint16_t>(u[e]);
						}
					}
				}
				continue;
			}
			// columns (0, 1) and (2, 3) of each row in paired FMAs: two
			// independent round-to-nearest FMAs per instruction, the same
			// results as four scalar ones
			float2 acc2[kGroup][2];
#pragma unroll
			for (int j = 0; j < kGroup; ++j)
				acc2[j][0] = acc2[j][1] = make_float2(init, init);
#pragma unroll
			for (int s = 0; s < VS; ++s) {
				const float4 x = *reinterpret_cast<const float4 *>(in + off[s] + 4 * q);
				const float2 x01 = make_float2(x.x, x.y), x23 = make_float2(x.z, x.w);
				float cj[kGroup];
				if constexpr (kGroup == 4) {
					const float4 c4 = reinterpret_cast<const float4 *>(cf)[s];
					cj[0] = c4.x;
					cj[1] = c4.y;
					cj[2] = c4.z;
					cj[3] = c4.w;
				} else {
					const float2 c2 = reinterpret_cast<const float2 *>(cf)[s];
					cj[0] = c2.x;
					cj[1] = c2.y;
				}
#pragma unroll
				for (int j = 0; j < kGroup; ++j) {
					const float2 cc = make_float2(cj[j], cj[j]);
					acc2[j][0] = __ffma2_rn(cc, x01, acc2[j][0]);
					acc2[j][1] = __ffma2_rn(cc, x23, acc2[j][1]);
				}
			}
			float acc[kGroup][4];
#pragma unroll
			for (int j = 0; j < kGroup; ++j) {
				acc[j][0] = acc2[j][0].x;
				acc[j][1] = acc2[j][0].y;
				acc[j][2] = acc2[j][1].x;
				acc[j][3] = acc2[j][1].y;
			}
#pragma unroll
			for (int j = 0; j < kGroup; ++j) {
				if (!FINAL) {
					float4 v;
					if (U16) {
						v.x = u16_round(acc[j][0], it.magic, it.pixel_max) - it.magic;
						v.y = u16_round(acc[j][1], it.magic, it.pixel_max) - it.magic;
						v.z = u16_round(acc[j][2], it.magic, it.pixel_max) - it.magic;
						v.w = u16_round(acc[j][3], it.magic, it.pixel_max) - it.magic;
					} else {
						v = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
					}
					*reinterpret_cast<float4 *>(I + (gi * kGroup + j) * i_pitch + 4 * q) = v;
				} else {
					const int r = g * kGroup + j;
					if (r >= it.dst_h)
						continue;
					const int x0 = 4 * q;
					char *drow = it.dst + static_cast<ptrdiff_t>(r) * it.dst_stride;
					if (U16) {
						uint32_t u[4];
#pragma unroll
						for (int e = 0; e < 4; ++e)
							u[e] = __float_as_uint(u16_round(acc[j][e], it.magic, it.pixel_max)) & 0xFFFFu;
						uint16_t *d = reinterpret_cast<uint16_t *>(drow) + it.c0 + x0;
						if (it.vec_ok && x0 + 3 < it.cols_valid) {
							*reinterpret_cast<uint2 *>(d) = make_uint2(u[0] | (u[1] << 16), u[2] | (u[3] << 16));
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < it.cols_valid)
									d[e] = static_cast<uint16_t>(u[e]);
						}
					} else {
						float *d = reinterpret_cast<float *>(drow) + it.c0 + x0;
						if (it.vec_ok && x0 + 3 < it.cols_valid) {
							*reinterpret_cast<float4 *>(d) = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < it.cols_valid)
									d[e] = acc[j][e];
						}
					}
				}
			}
		}
	}
}

// Source-line range a step needs: groups [g0, g1) read lines
// [base[g0], base[g1 - 1] + VS) (bases are non-decreasing).
template <int VS>
__device__ __forceinline__ int step_end(const Item &it, const char *smem, const SmemLayout &L, int g1)
{
	return reinterpret_cast<const int *>(smem + L.vbase_off)[g1 - 1 - it.g_begin] + VS;
}

template <int VS, int kGroup>
__device__ __forceinline__ void load_coef(const Item &it, int g0, int g1, char *dst)
{
	// kGroup floats per line: (g1 - g0) * VS * kGroup * 4 bytes, a multiple of 16 (VS even)
	const char *src = it.v_dense + static_cast<size_t>(g0) * VS * kGroup * 4;
	for (int i = threadIdx.x; i < (g1 - g0) * VS * kGroup / 4; i += kThreads)
		cp_async16(dst + i * 16, src + i * 16, 16);
}

template <bool H_FIRST, bool U16, int HW, int VS, bool INT = false>
__global__ void __launch_bounds__(kThreads, H_FIRST ? 4 : 5)
fused_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_items, const __grid_constant__ FusedJob single,
             const __grid_constant__ SmemLayout L, const __grid_constant__ WorkChunks C)
{
	constexpr int kGroup = group_rows(H_FIRST);
	extern __shared__ float4 smem4[];
	char *smem = reinterpret_cast<char *>(smem4);
	float *ring = reinterpret_cast<float *>(smem + L.ring_off);
	char *stage = smem + L.stage_off;
	float *in = reinterpret_cast<float *>(smem + L.in_off);
	float *I = reinterpret_cast<float *>(smem + L.i_off);
	const int rmask = L.ring_rows - 1;
	const int smask = L.stage_rows - 1;
	const int imask = L.in_rows - 1;

	// Lines a step reads but does not load keep finite values: clear the rings once.
	for (int i = threadIdx.x; i < L.vcoef_off / 16; i += kThreads)
		smem4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
	__syncthreads();

	// the launch's units in job / strip / step order: guided chunks
	// (C.sched), or this CTA's equal share
	__shared__ int chunk;
	int c_begin = static_cast<int>(static_cast<long long>(blockIdx.x) * total_items / gridDim.x);
	int c_end = static_cast<int>(static_cast<long long>(blockIdx.x + 1) * total_items / gridDim.x);
	for (bool first = true;; first = false) {
		if (C.sched) {
			const int m = next_chunk(C, &chunk);
			if (m < 0)
				break;
			c_begin = __ldg(C.bounds + m);
			c_end = __ldg(C.bounds + m + 1);
		} else if (!first) {
			break;
		}
		const int t_end = c_end;
		for (int t = c_begin; t < t_end;) {
			const FusedJob *Jp = jobs ? &jobs[find_job(jobs, num_jobs, t)] : &single;
			const Item it = make_item<HW>(*Jp, t, t_end, smem, L);
			t += it.units;
			__syncthreads();  // group bases visible

			const int nsteps = (it.g_end - it.g_begin + it.step_groups - 1) / it.step_groups;
			// step k covers groups [gk, gk1); its new source lines are [lo_k, hi_k)
			int hi_prev = reinterpret_cast<const int *>(smem + L.vbase_off)[0];
			auto step_groups_of = [&](int k, int *g0, int *g1) {
				*g0 = it.g_begin + k * it.step_groups;
				*g1 = min(it.g_end, *g0 + it.step_groups);
			};
			// prologue: step 0's lines and taps
			{
				int g0, g1;
				step_groups_of(0, &g0, &g1);
				const int hi = step_end<VS>(it, smem, L, g1);
				if (U16)
					load_lines<true>(it, hi_prev, hi, stage, smask, L.pitch);
				else
					load_lines<false>(it, hi_prev, hi, reinterpret_cast<char *>(H_FIRST ? in : ring),
					                  H_FIRST ? imask : rmask, L.pitch);
				load_coef<VS, kGroup>(it, g0, g1, smem + L.vcoef_off);
				cp_async_commit();
			}
			__syncthreads();  // lines stored by plain loads (unaligned u16) are visible to every converter
			int lo_cur = hi_prev;
			int hi_cur = step_end<VS>(it, smem, L, min(it.g_end, it.g_begin + it.step_groups));

			for (int k = 0; k < nsteps; ++k) {
				int g0, g1;
				step_groups_of(k, &g0, &g1);
				// prefetch step k+1
				int hi_next = hi_cur;
				if (k + 1 < nsteps) {
					int n0, n1;
					step_groups_of(k + 1, &n0, &n1);
					hi_next = step_end<VS>(it, smem, L, n1);
					if (U16)
						load_lines<true>(it, hi_cur, hi_next, stage, smask, L.pitch);
					else
						load_lines<false>(it, hi_cur, hi_next, reinterpret_cast<char *>(H_FIRST ? in : ring),
						                  H_FIRST ? imask : rmask, L.pitch);
					load_coef<VS, kGroup>(it, n0, n1, smem + L.vcoef_off + ((k + 1) & 1) * (L.vbase_off - L.vcoef_off) / 2);
				}
				cp_async_commit();
				cp_async_wait<1>();
				if (U16)
					convert_lines<INT>(it, lo_cur, hi_cur, stage, smask, H_FIRST ? in : ring, H_FIRST ? imask : rmask, L.pitch);
				__syncthreads();

				const float *coef = reinterpret_cast<const float *>(smem + L.vcoef_off + (k & 1) * (L.vbase_off - L.vcoef_off) / 2);
				if (H_FIRST) {
					// new source lines -> intermediate ring
					h_pass<U16, false, HW, INT>(it, smem, L, in, imask, lo_cur, hi_cur, ring, rmask, 0);
					__syncthreads();
					v_pass<U16, true, VS, kGroup, INT>(it, smem, L, ring, rmask, kStripW, g0, g1, coef, kStripW / 4, nullptr, 0);
				} else {
					v_pass<U16, false, VS, kGroup, INT>(it, smem, L, ring, rmask, L.pitch, g0, g1, coef, it.pxa / 4, I, L.pitch);
					__syncthreads();
					h_pass<U16, true, HW, INT>(it, smem, L, I, 0x7fffffff, 0, (g1 - g0) * kGroup, nullptr, 0, g0 * kGroup);
				}
				lo_cur = hi_cur;
				hi_cur = hi_next;
			}
			cp_async_wait<0>();
			__syncthreads();  // the next item reuses every buffer
		}
	}
	if (C.sched)
		chunks_finish(C);
}

} // namespace fused_detail
} // namespace zg
