// The fused two-pass tile kernel (template). Instantiated per variant in
// fused_inst_*.cu.
//
// Per output tile (tile_h x kTileW):
//   1. load the source patch  src[win_row] x src[win_col]  into shared memory
//      (u16 samples re-centred to exact floats on the way in);
//   2. first pass  (H for H-first, V for V-first) into a shared intermediate;
//   3. second pass from the intermediate straight to the destination plane.
// The intermediate never touches HBM. The grid is persistent: each CTA walks
// the batch's global tile list with a stride of gridDim.x.
#pragma once

#include "fused.h"

namespace zg {
namespace fused_detail {

constexpr int kTileW = 128;  // output columns per tile
constexpr int kThreads = kTileThreads;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ int find_job(const FusedJob *__restrict__ jobs, int num_jobs, int t)
{
	int lo = 0, hi = num_jobs - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (__ldg(&jobs[mid].tile_begin) <= t)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
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

__device__ __forceinline__ float u16_to_centred(uint32_t v, float bias)
{
	// v + 2^23 exactly, minus (2^23 + offset)
	return __int_as_float(0x4B000000 | v) - bias;
}

template <bool U16>
__device__ __forceinline__ void load_patch(const FusedJob &J, float *__restrict__ P, int pitch, int ylo, int py,
                                           int xlo, int pxa)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const char *base = static_cast<const char *>(J.src);
	if (!U16) {
		const int q = pxa >> 2;
		for (int r = warp; r < py; r += kWarps) {
			const int gy = ylo + r;
			const bool row_ok = gy < J.src_h;
			const float *row = reinterpret_cast<const float *>(base + static_cast<ptrdiff_t>(row_ok ? gy : 0) * J.src_stride);
			for (int qx = lane; qx < q; qx += 32) {
				const int gx = xlo + 4 * qx;
				float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
				if (row_ok) {
					if (J.vec_ok && gx + 3 < J.src_w) {
						v = __ldg(reinterpret_cast<const float4 *>(row + gx));
					} else {
						if (gx + 0 < J.src_w) v.x = __ldg(row + gx + 0);
						if (gx + 1 < J.src_w) v.y = __ldg(row + gx + 1);
						if (gx + 2 < J.src_w) v.z = __ldg(row + gx + 2);
						if (gx + 3 < J.src_w) v.w = __ldg(row + gx + 3);
					}
				}
				*reinterpret_cast<float4 *>(P + r * pitch + 4 * qx) = v;
			}
		}
	} else {
		const float bias = 8388608.0f + J.offset;
		const int q = pxa >> 3;
		for (int r = warp; r < py; r += kWarps) {
			const int gy = ylo + r;
			const bool row_ok = gy < J.src_h;
			const uint16_t *row = reinterpret_cast<const uint16_t *>(base + static_cast<ptrdiff_t>(row_ok ? gy : 0) * J.src_stride);
			for (int qx = lane; qx < q; qx += 32) {
				const int gx = xlo + 8 * qx;
				uint32_t w[4] = { 0, 0, 0, 0 };
				bool have[8];
				if (row_ok && J.vec_ok && gx + 7 < J.src_w) {
					uint4 u = __ldg(reinterpret_cast<const uint4 *>(row + gx));
					w[0] = u.x; w[1] = u.y; w[2] = u.z; w[3] = u.w;
#pragma unroll
					for (int i = 0; i < 8; ++i)
						have[i] = true;
				} else {
#pragma unroll
					for (int i = 0; i < 8; ++i) {
						have[i] = row_ok && gx + i < J.src_w;
						if (have[i])
							w[i >> 1] |= static_cast<uint32_t>(__ldg(row + gx + i)) << (16 * (i & 1));
					}
				}
				float f[8];
#pragma unroll
				for (int i = 0; i < 8; ++i) {
					const uint32_t v = (w[i >> 1] >> (16 * (i & 1))) & 0xFFFFu;
					// samples outside the plane are never weighted; keep them finite
					f[i] = have[i] ? u16_to_centred(v, bias) : 0.0f;
				}
				float *dst = P + r * pitch + 8 * qx;
				*reinterpret_cast<float4 *>(dst) = make_float4(f[0], f[1], f[2], f[3]);
				*reinterpret_cast<float4 *>(dst + 4) = make_float4(f[4], f[5], f[6], f[7]);
			}
		}
	}
}

// Horizontal pass on shared memory: out[y][c] = sum_k taps[c][k] * in[y][left[c] + k].
// One thread per output column (taps in registers), rows strided by the CTA.
// FINAL: write the destination plane; else write the shared intermediate.
template <bool U16, bool FINAL, int HW>
__device__ __forceinline__ void h_pass(const FusedJob &J, const float *__restrict__ in, int in_pitch, int rows,
                                       int xlo, int c0, int out_rows_valid, float *__restrict__ I, int i_pitch,
                                       int r0)
{
	const int c = threadIdx.x % kTileW;
	const int gc = c0 + c;
	const bool col_ok = gc < J.dst_w;
	float taps[HW];
	int l = 0;
	if (col_ok) {
		const float4 *tp = reinterpret_cast<const float4 *>(J.h_taps + static_cast<size_t>(gc) * HW);
#pragma unroll
		for (int k = 0; k < HW / 4; ++k) {
			float4 t4 = __ldg(tp + k);
			taps[4 * k] = t4.x; taps[4 * k + 1] = t4.y; taps[4 * k + 2] = t4.z; taps[4 * k + 3] = t4.w;
		}
		l = __ldg(J.h_left + gc) - xlo;
	} else {
#pragma unroll
		for (int k = 0; k < HW; ++k)
			taps[k] = 0.0f;
	}
	const float init = U16 ? 8192.0f : 0.0f;
	for (int y = threadIdx.x / kTileW; y < rows; y += kThreads / kTileW) {
		const float *row = in + y * in_pitch + l;
		float acc = init;
#pragma unroll
		for (int k = 0; k < HW; ++k)
			acc = __fmaf_rn(taps[k], row[k], acc);
		if (!FINAL) {
			float v = acc;
			if (U16)
				v = u16_round(acc, J.magic, J.pixel_max) - J.magic;
			I[y * i_pitch + c] = v;
		} else if (col_ok && y < out_rows_valid) {
			char *drow = static_cast<char *>(J.dst) + static_cast<ptrdiff_t>(r0 + y) * J.dst_stride;
			if (U16) {
				const float q = u16_round(acc, J.magic, J.pixel_max);
				reinterpret_cast<uint16_t *>(drow)[gc] = static_cast<uint16_t>(__float_as_uint(q) & 0xFFFFu);
			} else {
				reinterpret_cast<float *>(drow)[gc] = acc;
			}
		}
	}
}

// Vertical pass on shared memory with dense groups of kGroup output rows:
// out[g*4 + j][x] = sum_s dense[g][s][j] * in[base[g] - ylo + s][x], four
// adjacent columns per thread (16-byte shared loads).
template <bool U16, bool FINAL, int VS>
__device__ __forceinline__ void v_pass(const FusedJob &J, const float *__restrict__ in, int in_pitch, int ylo,
                                       int groups, int g0, int quads, float *__restrict__ I, int i_pitch, int r0,
                                       int c0, int out_rows_valid, int out_cols_valid)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const float init = U16 ? 8192.0f : 0.0f;
	for (int g = warp; g < groups; g += kWarps) {
		const int gg = g0 + g;
		const int base = __ldg(J.v_base + gg) - ylo;
		const float4 *dense = reinterpret_cast<const float4 *>(J.v_dense) + static_cast<size_t>(gg) * VS;
		for (int qx = lane; qx < quads; qx += 32) {
			float acc[kGroup][4];
#pragma unroll
			for (int j = 0; j < kGroup; ++j)
#pragma unroll
				for (int e = 0; e < 4; ++e)
					acc[j][e] = init;
			const float *col = in + base * in_pitch + 4 * qx;
#pragma unroll
			for (int s = 0; s < VS; ++s) {
				const float4 x = *reinterpret_cast<const float4 *>(col + s * in_pitch);
				const float4 cf = __ldg(dense + s);
				const float cj[4] = { cf.x, cf.y, cf.z, cf.w };
#pragma unroll
				for (int j = 0; j < kGroup; ++j) {
					acc[j][0] = __fmaf_rn(cj[j], x.x, acc[j][0]);
					acc[j][1] = __fmaf_rn(cj[j], x.y, acc[j][1]);
					acc[j][2] = __fmaf_rn(cj[j], x.z, acc[j][2]);
					acc[j][3] = __fmaf_rn(cj[j], x.w, acc[j][3]);
				}
			}
#pragma unroll
			for (int j = 0; j < kGroup; ++j) {
				const int r = g * kGroup + j;
				if (!FINAL) {
					float4 v;
					if (U16) {
						v.x = u16_round(acc[j][0], J.magic, J.pixel_max) - J.magic;
						v.y = u16_round(acc[j][1], J.magic, J.pixel_max) - J.magic;
						v.z = u16_round(acc[j][2], J.magic, J.pixel_max) - J.magic;
						v.w = u16_round(acc[j][3], J.magic, J.pixel_max) - J.magic;
					} else {
						v = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
					}
					*reinterpret_cast<float4 *>(I + r * i_pitch + 4 * qx) = v;
				} else if (r < out_rows_valid) {
					const int x0 = 4 * qx;
					char *drow = static_cast<char *>(J.dst) + static_cast<ptrdiff_t>(r0 + r) * J.dst_stride;
					if (U16) {
						uint32_t q[4];
#pragma unroll
						for (int e = 0; e < 4; ++e)
							q[e] = __float_as_uint(u16_round(acc[j][e], J.magic, J.pixel_max)) & 0xFFFFu;
						uint16_t *d = reinterpret_cast<uint16_t *>(drow) + c0 + x0;
						if (J.vec_ok && x0 + 3 < out_cols_valid) {
							*reinterpret_cast<uint2 *>(d) = make_uint2(q[0] | (q[1] << 16), q[2] | (q[3] << 16));
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < out_cols_valid)
									d[e] = static_cast<uint16_t>(q[e]);
						}
					} else {
						float *d = reinterpret_cast<float *>(drow) + c0 + x0;
						if (J.vec_ok && x0 + 3 < out_cols_valid) {
							*reinterpret_cast<float4 *>(d) = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < out_cols_valid)
									d[e] = acc[j][e];
						}
					}
				}
			}
		}
	}
}

template <bool H_FIRST, bool U16, int HW, int VS>
__global__ void __launch_bounds__(kThreads, 2)
fused_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_tiles, const __grid_constant__ FusedJob single)
{
	extern __shared__ float4 smem4[];
	float *smem = reinterpret_cast<float *>(smem4);

	for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
		const FusedJob &J = jobs ? jobs[find_job(jobs, num_jobs, t)] : single;
		const int local = t - J.tile_begin;
		const int ty = local / J.tiles_x, tx = local - ty * J.tiles_x;
		const int r0 = ty * J.tile_h, c0 = tx * kTileW;
		const int rows_valid = min(J.tile_h, J.dst_h - r0);
		const int cols_valid = min(kTileW, J.dst_w - c0);
		const int ylo = __ldg(J.win_row + 2 * ty), yhi = __ldg(J.win_row + 2 * ty + 1);
		const int xlo = __ldg(J.win_col + 2 * tx), xhi = __ldg(J.win_col + 2 * tx + 1);
		const int py = yhi - ylo;
		const int pxa = (xhi - xlo + 7) & ~7;   // multiple of 8 columns
		const int p_pitch = pxa + 4;            // keeps row starts 16-byte aligned
		float *P = smem;
		float *I = smem + py * p_pitch;
		const int groups = J.tile_h / kGroup;

		__syncthreads();  // the previous tile is done with shared memory
		load_patch<U16>(J, P, p_pitch, ylo, py, xlo, pxa);
		__syncthreads();
		if (H_FIRST) {
			// H: all patch rows, the tile's columns -> I[py][kTileW]
			h_pass<U16, false, HW>(J, P, p_pitch, py, xlo, c0, 0, I, kTileW, 0);
			__syncthreads();
			// V: I -> destination
			v_pass<U16, true, VS>(J, I, kTileW, ylo, groups, r0 / kGroup, kTileW / 4, nullptr, 0, r0, c0, rows_valid,
			                      cols_valid);
		} else {
			// V: tile rows, all patch columns -> I[tile_h][pxa]
			v_pass<U16, false, VS>(J, P, p_pitch, ylo, groups, r0 / kGroup, pxa / 4, I, p_pitch, r0, c0, 0, 0);
			__syncthreads();
			// H: I -> destination
			h_pass<U16, true, HW>(J, I, p_pitch, J.tile_h, xlo, c0, rows_valid, nullptr, 0, r0);
		}
	}
}

} // namespace fused_detail
} // namespace zg
