// The fused two-pass tile kernel (template). Instantiated per variant in
// fused_inst_*.cu.
//
// Per output tile (tile_h x kTileW):
//   1. the tile's source patch src[win_row] x src[win_col], its vertical tap
//      groups, horizontal taps and window tables arrive in shared memory by
//      cp.async, issued while the CTA was still computing the previous tile
//      (two buffers);
//   2. u16 samples are re-centred to exact floats;
//   3. first pass  (H for H-first, V for V-first) into a shared intermediate;
//   4. second pass from the intermediate straight to the destination plane.
// The intermediate never touches HBM. The grid is persistent: each CTA walks
// the launch's global tile list with a stride of gridDim.x.
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

// ------------------------------------------------------------ async copies --
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

// Everything one tile needs, resolved from the job table.
struct Tile {
	int job;
	int r0, c0, ty, tx;
	int rows_valid, cols_valid;
	int ylo, py, xlo, pxa, pitch;
	int tile_h, vec_ok;
	char *dst;
	ptrdiff_t dst_stride;
	float magic, pixel_max, offset;
};

__device__ __forceinline__ Tile make_tile(const FusedJob &J, int job, int t)
{
	Tile T;
	T.job = job;
	const int local = t - J.tile_begin;
	T.ty = local / J.tiles_x;
	T.tx = local - T.ty * J.tiles_x;
	T.r0 = T.ty * J.tile_h;
	T.c0 = T.tx * kTileW;
	T.rows_valid = min(J.tile_h, J.dst_h - T.r0);
	T.cols_valid = min(kTileW, J.dst_w - T.c0);
	T.ylo = __ldg(J.win_row + 2 * T.ty);
	T.py = __ldg(J.win_row + 2 * T.ty + 1) - T.ylo;
	T.xlo = __ldg(J.win_col + 2 * T.tx);
	T.pxa = (__ldg(J.win_col + 2 * T.tx + 1) - T.xlo + 7) & ~7;
	T.pitch = T.pxa + 8;
	T.tile_h = J.tile_h;
	T.vec_ok = J.vec_ok;
	T.dst = static_cast<char *>(J.dst);
	T.dst_stride = J.dst_stride;
	T.magic = J.magic;
	T.pixel_max = J.pixel_max;
	T.offset = J.offset;
	return T;
}

// Issue the async copies of one tile into buffer `buf`:
//   patch (source samples, zero outside the plane), v-group taps, h taps,
//   h left offsets, v group bases.
template <bool U16, int HW, int VS>
__device__ __forceinline__ void prefetch_tile(const FusedJob &J, const Tile &T, char *buf, const SmemLayout &L)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	constexpr int E = U16 ? 2 : 4;          // bytes per sample
	constexpr int PER = 16 / E;             // samples per 16-byte chunk
	const char *src = static_cast<const char *>(J.src);
	char *patch = buf;
	const int chunks = T.pxa / PER;
	const int row_bytes = T.pitch * E;
	for (int r = warp; r < T.py; r += kWarps) {
		const int gy = T.ylo + r;
		const bool row_ok = gy < J.src_h;
		const char *row = src + static_cast<ptrdiff_t>(row_ok ? gy : 0) * J.src_stride;
		char *srow = patch + r * row_bytes;
		if (J.vec_ok) {
			for (int q = lane; q < chunks; q += 32) {
				const int gx = T.xlo + q * PER;
				int n = row_ok ? min(PER, J.src_w - gx) : 0;
				n = max(n, 0);
				cp_async16(srow + q * 16, n ? row + static_cast<ptrdiff_t>(gx) * E : src, n * E);
			}
		} else if (!U16) {
			for (int x = lane; x < T.pxa; x += 32) {
				const int gx = T.xlo + x;
				const bool ok = row_ok && gx < J.src_w;
				cp_async4(srow + x * 4, ok ? row + static_cast<ptrdiff_t>(gx) * 4 : src, ok ? 4 : 0);
			}
		} else {
			// 2-byte samples at 2-byte alignment: plain loads
			for (int x = lane; x < T.pxa; x += 32) {
				const int gx = T.xlo + x;
				const bool ok = row_ok && gx < J.src_w;
				reinterpret_cast<uint16_t *>(srow)[x] = ok ? __ldg(reinterpret_cast<const uint16_t *>(row) + gx) : 0;
			}
		}
	}
	// v-group taps: groups [r0/4, r0/4 + tile_h/4), VS float4 each
	const int groups = J.tile_h / kGroup;
	const char *vd = reinterpret_cast<const char *>(J.v_dense) + static_cast<size_t>(T.r0 / kGroup) * VS * 16;
	for (int i = threadIdx.x; i < groups * VS; i += kThreads)
		cp_async16(buf + L.vcoef_off + i * 16, vd + i * 16, 16);
	// h taps of the tile's columns (zero past the plane)
	const char *ht = reinterpret_cast<const char *>(J.h_taps) + static_cast<size_t>(T.c0) * HW * 4;
	for (int i = threadIdx.x; i < kTileW * HW / 4; i += kThreads) {
		const int col = (i * 4) / HW;
		cp_async16(buf + L.htaps_off + i * 16, col < T.cols_valid ? ht + i * 16 : ht, col < T.cols_valid ? 16 : 0);
	}
	for (int i = threadIdx.x; i < kTileW / 4; i += kThreads) {
		const int n = max(0, min(4, T.cols_valid - 4 * i));
		cp_async16(buf + L.hleft_off + i * 16, n ? J.h_left + T.c0 + 4 * i : J.h_left, n * 4);
	}
	for (int i = threadIdx.x; i < groups / 4; i += kThreads)
		cp_async16(buf + L.vbase_off + i * 16, J.v_base + T.r0 / kGroup + 4 * i, 16);
}

// u16 patch (raw samples in buf) -> centred floats in Pf.
__device__ __forceinline__ void convert_u16(const Tile &T, const char *buf, float *Pf, float offset)
{
	const float bias = 8388608.0f + offset;
	const int chunks = T.pxa / 8;
	for (int i = threadIdx.x; i < T.py * chunks; i += kThreads) {
		const int r = i / chunks, q = i - r * chunks;
		const uint4 u = *reinterpret_cast<const uint4 *>(buf + r * T.pitch * 2 + q * 16);
		const uint32_t w[4] = { u.x, u.y, u.z, u.w };
		float f[8];
#pragma unroll
		for (int k = 0; k < 8; ++k) {
			const uint32_t v = (w[k >> 1] >> (16 * (k & 1))) & 0xFFFFu;
			f[k] = __int_as_float(0x4B000000 | v) - bias;
		}
		float *d = Pf + r * T.pitch + q * 8;
		*reinterpret_cast<float4 *>(d) = make_float4(f[0], f[1], f[2], f[3]);
		*reinterpret_cast<float4 *>(d + 4) = make_float4(f[4], f[5], f[6], f[7]);
	}
}

// Horizontal pass: out[y][c] = sum_k taps[c][k] * in[y][left[c] - xlo + k].
// One thread per output column (taps in registers), rows strided by the CTA.
template <bool U16, bool FINAL, int HW>
__device__ __forceinline__ void h_pass(const Tile &T, const char *buf, const SmemLayout &L,
                                       const float *__restrict__ in, int in_pitch, int rows, float *__restrict__ I,
                                       int i_pitch)
{
	const int c = threadIdx.x % kTileW;
	const bool col_ok = c < T.cols_valid;
	float taps[HW];
	const float4 *tp = reinterpret_cast<const float4 *>(buf + L.htaps_off) + c * (HW / 4);
#pragma unroll
	for (int k = 0; k < HW / 4; ++k) {
		const float4 t4 = tp[k];
		taps[4 * k] = t4.x;
		taps[4 * k + 1] = t4.y;
		taps[4 * k + 2] = t4.z;
		taps[4 * k + 3] = t4.w;
	}
	const int l = col_ok ? reinterpret_cast<const int *>(buf + L.hleft_off)[c] - T.xlo : 0;
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
				v = u16_round(acc, T.magic, T.pixel_max) - T.magic;
			I[y * i_pitch + c] = v;
		} else if (col_ok && y < T.rows_valid) {
			char *drow = T.dst + static_cast<ptrdiff_t>(T.r0 + y) * T.dst_stride;
			if (U16) {
				const float q = u16_round(acc, T.magic, T.pixel_max);
				reinterpret_cast<uint16_t *>(drow)[T.c0 + c] = static_cast<uint16_t>(__float_as_uint(q) & 0xFFFFu);
			} else {
				reinterpret_cast<float *>(drow)[T.c0 + c] = acc;
			}
		}
	}
}

// Vertical pass with dense groups of kGroup output rows:
// out[g*4 + j][x] = sum_s dense[g][s][j] * in[base[g] - ylo + s][x], four
// adjacent columns per thread (16-byte shared loads, broadcast tap loads).
template <bool U16, bool FINAL, int VS>
__device__ __forceinline__ void v_pass(const Tile &T, const char *buf, const SmemLayout &L,
                                       const float *__restrict__ in, int in_pitch, int quads, float *__restrict__ I,
                                       int i_pitch)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const float init = U16 ? 8192.0f : 0.0f;
	const int groups = T.tile_h / kGroup;
	const float4 *dense_all = reinterpret_cast<const float4 *>(buf + L.vcoef_off);
	const int *vbase = reinterpret_cast<const int *>(buf + L.vbase_off);
	for (int g = warp; g < groups; g += kWarps) {
		const int base = vbase[g] - T.ylo;
		const float4 *dense = dense_all + g * VS;
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
				const float4 cf = dense[s];
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
						v.x = u16_round(acc[j][0], T.magic, T.pixel_max) - T.magic;
						v.y = u16_round(acc[j][1], T.magic, T.pixel_max) - T.magic;
						v.z = u16_round(acc[j][2], T.magic, T.pixel_max) - T.magic;
						v.w = u16_round(acc[j][3], T.magic, T.pixel_max) - T.magic;
					} else {
						v = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
					}
					*reinterpret_cast<float4 *>(I + r * i_pitch + 4 * qx) = v;
				} else if (r < T.rows_valid) {
					const int x0 = 4 * qx;
					char *drow = T.dst + static_cast<ptrdiff_t>(T.r0 + r) * T.dst_stride;
					if (U16) {
						uint32_t q[4];
#pragma unroll
						for (int e = 0; e < 4; ++e)
							q[e] = __float_as_uint(u16_round(acc[j][e], T.magic, T.pixel_max)) & 0xFFFFu;
						uint16_t *d = reinterpret_cast<uint16_t *>(drow) + T.c0 + x0;
						if (T.vec_ok && x0 + 3 < T.cols_valid) {
							*reinterpret_cast<uint2 *>(d) = make_uint2(q[0] | (q[1] << 16), q[2] | (q[3] << 16));
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < T.cols_valid)
									d[e] = static_cast<uint16_t>(q[e]);
						}
					} else {
						float *d = reinterpret_cast<float *>(drow) + T.c0 + x0;
						if (T.vec_ok && x0 + 3 < T.cols_valid) {
							*reinterpret_cast<float4 *>(d) = make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
						} else {
#pragma unroll
							for (int e = 0; e < 4; ++e)
								if (x0 + e < T.cols_valid)
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
fused_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_tiles, const __grid_constant__ FusedJob single,
             const __grid_constant__ SmemLayout L)
{
	extern __shared__ float4 smem4[];
	char *smem = reinterpret_cast<char *>(smem4);

	int t = blockIdx.x;
	if (t >= total_tiles)
		return;
	const FusedJob *Jp = jobs ? &jobs[find_job(jobs, num_jobs, t)] : &single;
	Tile T = make_tile(*Jp, 0, t);
	prefetch_tile<U16, HW, VS>(*Jp, T, smem, L);
	cp_async_commit();

	for (int it = 0; t < total_tiles; ++it, t += gridDim.x) {
		char *buf = smem + (it & 1) * L.buf_bytes;
		// prefetch the next tile of this CTA into the other buffer
		const int tn = t + gridDim.x;
		Tile Tn;
		if (tn < total_tiles) {
			const FusedJob *Jn = jobs ? &jobs[find_job(jobs, num_jobs, tn)] : &single;
			Tn = make_tile(*Jn, 0, tn);
			prefetch_tile<U16, HW, VS>(*Jn, Tn, smem + ((it + 1) & 1) * L.buf_bytes, L);
		}
		cp_async_commit();
		cp_async_wait<1>();
		__syncthreads();

		const float *P;
		if (U16) {
			float *Pf = reinterpret_cast<float *>(smem + L.pf_off);
			convert_u16(T, buf, Pf, T.offset);
			__syncthreads();
			P = Pf;
		} else {
			P = reinterpret_cast<const float *>(buf);
		}
		float *I = reinterpret_cast<float *>(smem + L.i_off);
		if (H_FIRST) {
			h_pass<U16, false, HW>(T, buf, L, P, T.pitch, T.py, I, kTileW);
			__syncthreads();
			v_pass<U16, true, VS>(T, buf, L, I, kTileW, kTileW / 4, nullptr, 0);
		} else {
			v_pass<U16, false, VS>(T, buf, L, P, T.pitch, T.pxa / 4, I, T.pitch);
			__syncthreads();
			h_pass<U16, true, HW>(T, buf, L, I, T.pitch, T.tile_h, nullptr, 0);
		}
		__syncthreads();  // this buffer and I are free for the next iteration
		if (tn < total_tiles)
			T = Tn;
	}
	cp_async_wait<0>();
}

} // namespace fused_detail
} // namespace zg
