// Depth conversion of one plane (zimg's DepthConversion, src/zimg/depth/):
// left shift, integer to FLOAT or HALF, HALF <-> FLOAT, and dither (NONE /
// ORDERED / RANDOM) to an integer type. One pass over the plane, HBM-bound:
// each thread converts runs of 8 samples of one line with vector loads and
// stores where the plane allows. Error diffusion is ed_kernel.cu.
//
// Arithmetic is zimg's C path in IEEE single precision, step for step:
// x * scale rounded, + offset rounded (no fused multiply-add,
// depth_convert.cpp:32-39, dither.cpp:45-49), + dither value rounded, clamp
// to [0, 2^depth - 1], round to nearest even (lrint under the default
// rounding mode).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "depth.h"
#include "depth_device.cuh"

namespace zg {

namespace {

constexpr int kRun = 8;         // samples per thread per step
constexpr int kThreads = 256;

// zimg's 16x16 ordered-dither matrix (dither.cpp:137-155) from its recursive
// definition: digit k of row i and column j adds B[bit_k(i)][bit_k(j)] *
// 4^(3-k), B = {{0, 3}, {2, 1}}.
__device__ __forceinline__ unsigned bayer16(unsigned i, unsigned j)
{
	unsigned v = 0;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const unsigned bi = (i >> k) & 1, bj = (j >> k) & 1;
		const unsigned digit = bi ? (bj ? 1u : 2u) : (bj ? 3u : 0u);
		v += digit << (2 * (3 - k));
	}
	return v;
}

// zimg's 64 x 64 blue-noise matrix (blue.h:10-13), four row-major entries
// per little-endian word.
__device__ const uint32_t kBlueNoiseWords[1024] = {
#include "blue_noise_table.inc"
};

// binary32 -> binary16 bits, rounded to nearest even; overflow to infinity;
// NaNs keep the payload's top bits with the quiet bit set.
__device__ __forceinline__ uint32_t float_to_half_bits(float f)
{
	const uint32_t x = __float_as_uint(f);
	const uint32_t sign = (x >> 16) & 0x8000u;
	const uint32_t e = (x >> 23) & 0xFFu, m = x & 0x7FFFFFu;
	if (e == 0xFFu)
		return sign | 0x7C00u | (m ? ((m >> 13) | 0x200u) : 0u);
	uint32_t sig = m, shift = 13, he;
	if (e <= 112u) {
		shift = min(13u + 112u - e + 1u, 31u);
		sig = m | 0x800000u;
		he = 0;
	} else {
		he = e - 112u;
	}
	const uint32_t rem = sig & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
	uint32_t q = sig >> shift;
	if (rem > halfway || (rem == halfway && (q & 1u)))
		++q;
	if (q > 0x3FFu) {
		q &= 0x3FFu;
		++he;
	}
	if (he >= 0x1Fu)
		return sign | 0x7C00u;
	return sign | (he << 10) | q;
}

template <class T>
__device__ __forceinline__ void load_run(const T *p, float (&x)[kRun], bool vec)
{
	if constexpr (std::is_same_v<T, Half>) {
		if (vec) {
			const uint4 v = *reinterpret_cast<const uint4 *>(p);
			const uint32_t w[4] = { v.x, v.y, v.z, v.w };
#pragma unroll
			for (int e = 0; e < kRun; ++e)
				x[e] = half_bits_to_float((w[e >> 1] >> (16 * (e & 1))) & 0xffffu);
		} else {
#pragma unroll
			for (int e = 0; e < kRun; ++e)
				x[e] = half_bits_to_float(p[e].bits);
		}
	} else if (vec) {
		if constexpr (sizeof(T) == 1) {
			const uint2 v = *reinterpret_cast<const uint2 *>(p);
			const uint32_t w[2] = { v.x, v.y };
#pragma unroll
			for (int e = 0; e < kRun; ++e)
				x[e] = static_cast<float>((w[e >> 2] >> (8 * (e & 3))) & 0xffu);
		} else if constexpr (sizeof(T) == 2) {
			const uint4 v = *reinterpret_cast<const uint4 *>(p);
			const uint32_t w[4] = { v.x, v.y, v.z, v.w };
#pragma unroll
			for (int e = 0; e < kRun; ++e)
				x[e] = static_cast<float>((w[e >> 1] >> (16 * (e & 1))) & 0xffffu);
		} else {
			const float4 a = reinterpret_cast<const float4 *>(p)[0];
			const float4 b = reinterpret_cast<const float4 *>(p)[1];
			x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
			x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
		}
	} else {
#pragma unroll
		for (int e = 0; e < kRun; ++e)
			x[e] = static_cast<float>(p[e]);
	}
}

// one sample of a partial run
template <class T>
__device__ __forceinline__ float load_one(const T *p)
{
	if constexpr (std::is_same_v<T, Half>)
		return half_bits_to_float(p->bits);
	else
		return static_cast<float>(*p);
}

// Round-to-nearest-even integers of 0 <= v < 2^22: v + 1.5 * 2^23 has an ulp
// of 1, so the sum's low mantissa bits are the rounded value (the same
// result as lrint under the default rounding mode).
__device__ __forceinline__ uint32_t round_bits(float v)
{
	return __float_as_uint(__fadd_rn(v, 12582912.0f));
}

// Eight rounded values (low bits of r) -> packed samples.
template <class U>
__device__ __forceinline__ void store_run(U *p, const uint32_t (&r)[kRun], int n, bool vec)
{
	if (vec && n == kRun) {
		if constexpr (sizeof(U) == 1) {
			// low bytes of four registers: two pairs, then the pairs
			const uint32_t a0 = __byte_perm(r[0], r[1], 0x5140), a1 = __byte_perm(r[2], r[3], 0x5140);
			const uint32_t b0 = __byte_perm(r[4], r[5], 0x5140), b1 = __byte_perm(r[6], r[7], 0x5140);
			*reinterpret_cast<uint2 *>(p) = make_uint2(__byte_perm(a0, a1, 0x5410), __byte_perm(b0, b1, 0x5410));
		} else {
			*reinterpret_cast<uint4 *>(p) =
				make_uint4(__byte_perm(r[0], r[1], 0x5410), __byte_perm(r[2], r[3], 0x5410),
				           __byte_perm(r[4], r[5], 0x5410), __byte_perm(r[6], r[7], 0x5410));
		}
	} else {
		for (int e = 0; e < n; ++e)
			p[e] = static_cast<U>(r[e] & (sizeof(U) == 1 ? 0xffu : 0xffffu));
	}
}

// MODE 1: left shift; 2: to float; 3: dither to integer. DITHER (MODE 3):
// 0 none, 1 ordered, 2 random.
template <class T, class U, int MODE, int DITHER>
__global__ void __launch_bounds__(kThreads)
depth_kernel(DepthLaunch L)
{
	// ORDERED: this plane's 16 x 16 dither values, row-major. RANDOM: the
	// values (m + 1) / 257 - 1/2 of the 256 matrix entries m, and the
	// plane's 64 x 64 entries already moved by its offsets, four per word.
	__shared__ __align__(16) float table[DITHER == 1 ? 256 : (DITHER == 2 ? 256 : 4)];
	__shared__ __align__(16) uint32_t noise[DITHER == 2 ? 1024 : 1];
	if (MODE == 3 && DITHER == 1) {
		for (int t = threadIdx.x; t < 256; t += kThreads) {
			const unsigned i = t >> 4, j = t & 15;
			// variants by plane (dither.cpp:170-186): as is, mirrored
			// left-right, top-bottom, transposed
			const unsigned s = L.seq & 3;
			const unsigned ii = s == 2 ? 15 - i : (s == 3 ? j : i);
			const unsigned jj = s == 1 ? 15 - j : (s == 3 ? i : j);
			// (m + 1) / 257 - 1/2 in float (dither.cpp:157-167)
			table[t] = __fsub_rn(__fdiv_rn(static_cast<float>(bayer16(ii, jj) + 1), 257.0f), 0.5f);
		}
		__syncthreads();
	}
	if (MODE == 3 && DITHER == 2) {
		for (int t = threadIdx.x; t < 256; t += kThreads)
			table[t] = __fsub_rn(__fdiv_rn(static_cast<float>(t + 1), 257.0f), 0.5f);
		// entry (line + voff, column + hoff) mod 64, (hoff, voff) by plane
		// (dither.cpp:226-233); hoff is a multiple of 4, so rows rotate by
		// whole words
		const unsigned s = L.seq & 3;
		const unsigned hoff = s == 1 ? 32 : (s == 2 ? 16 : (s == 3 ? 48 : 0));
		const unsigned voff = s == 1 ? 12 : (s == 2 ? 55 : (s == 3 ? 26 : 0));
		for (int t = threadIdx.x; t < 1024; t += kThreads) {
			const unsigned i = t >> 4, wj = t & 15;
			noise[t] = kBlueNoiseWords[((i + voff) & 63) * 16 + ((wj + hoff / 4) & 15)];
		}
		__syncthreads();
	}
	// the plane's runs of 8 samples, line by line, strided over the grid;
	// (line, run) advance by the stride's fixed quotient and remainder
	const int runs = (L.width + kRun - 1) / kRun;
	const long long total = static_cast<long long>(runs) * L.height;
	const long long stride = static_cast<long long>(gridDim.x) * kThreads;
	long long u = static_cast<long long>(blockIdx.x) * kThreads + threadIdx.x;
	int i = static_cast<int>(u / runs), r = static_cast<int>(u % runs);
	const int di = static_cast<int>(stride / runs), dr = static_cast<int>(stride % runs);
	for (; u < total; u += stride) {
		{
			const T *srow = reinterpret_cast<const T *>(static_cast<const char *>(L.src) + static_cast<ptrdiff_t>(i) * L.src_stride);
			U *drow = reinterpret_cast<U *>(static_cast<char *>(L.dst) + static_cast<ptrdiff_t>(i) * L.dst_stride);
			const float *trow = table + ((i & 15) << 4);
			const int j0 = r * kRun;
			const int n = min(kRun, L.width - j0);
			const T *s = srow + j0;
			U *d = drow + j0;
			float x[kRun];
			if (n == kRun) {
				load_run<T>(s, x, L.vec_in);
			} else {
#pragma unroll
				for (int e = 0; e < kRun; ++e)
					x[e] = e < n ? load_one<T>(s + e) : 0.0f;
			}
			if constexpr (MODE == 2) {
				// integer in: x * scale + offset; HALF / FLOAT in: the value
				// as it is (depth_convert.cpp:23-57)
				constexpr bool kFloatIn = std::is_same_v<T, float> || std::is_same_v<T, Half>;
				float y[kRun];
#pragma unroll
				for (int e = 0; e < kRun; ++e)
					y[e] = kFloatIn ? x[e] : __fadd_rn(__fmul_rn(x[e], L.scale), L.offset);
				if constexpr (std::is_same_v<U, Half>) {
					uint32_t h[kRun];
#pragma unroll
					for (int e = 0; e < kRun; ++e)
						h[e] = float_to_half_bits(y[e]);
					if (n == kRun && L.vec_out) {
						*reinterpret_cast<uint4 *>(d) = make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16),
						                                           h[4] | (h[5] << 16), h[6] | (h[7] << 16));
					} else {
						for (int e = 0; e < n; ++e)
							d[e].bits = static_cast<uint16_t>(h[e]);
					}
				} else if (n == kRun && L.vec_out) {
					reinterpret_cast<float4 *>(d)[0] = make_float4(y[0], y[1], y[2], y[3]);
					reinterpret_cast<float4 *>(d)[1] = make_float4(y[4], y[5], y[6], y[7]);
				} else {
					for (int e = 0; e < n; ++e)
						reinterpret_cast<float *>(d)[e] = y[e];
				}
			} else {
				uint32_t q[kRun];
				if constexpr (MODE == 1) {
#pragma unroll
					for (int e = 0; e < kRun; ++e)
						q[e] = static_cast<uint32_t>(x[e]) << L.shift;
				} else {
					// the run's 8 dither values: j0 is a multiple of 8
					float dv[kRun];
					if constexpr (DITHER == 1) {
						const float4 t0 = *reinterpret_cast<const float4 *>(trow + (j0 & 15));
						const float4 t1 = *reinterpret_cast<const float4 *>(trow + (j0 & 15) + 4);
						dv[0] = t0.x; dv[1] = t0.y; dv[2] = t0.z; dv[3] = t0.w;
						dv[4] = t1.x; dv[5] = t1.y; dv[6] = t1.z; dv[7] = t1.w;
					} else if constexpr (DITHER == 2) {
						const uint2 m8 = *reinterpret_cast<const uint2 *>(noise + (i & 63) * 16 + ((j0 & 63) >> 2));
#pragma unroll
						for (int e = 0; e < kRun; ++e)
							dv[e] = table[((e < 4 ? m8.x : m8.y) >> (8 * (e & 3))) & 0xFFu];
					} else {
#pragma unroll
						for (int e = 0; e < kRun; ++e)
							dv[e] = 0.0f;
					}
#pragma unroll
					for (int e = 0; e < kRun; ++e) {
						float v = __fadd_rn(__fmul_rn(x[e], L.scale), L.offset);
						v = __fadd_rn(v, dv[e]);
						v = fminf(fmaxf(v, 0.0f), L.vmax);
						q[e] = round_bits(v);
					}
				}
				store_run<U>(d, q, n, L.vec_out);
			}
		}
		r += dr;
		i += di;
		if (r >= runs) {
			r -= runs;
			++i;
		}
	}
}

template <class T>
constexpr bool is_int = std::is_same_v<T, uint8_t> || std::is_same_v<T, uint16_t>;
template <class T>
constexpr bool is_fp = std::is_same_v<T, float> || std::is_same_v<T, Half>;

template <class T, class U>
cudaError_t launch_tu(int mode, const DepthLaunch &L, int grid, cudaStream_t st)
{
	switch (mode) {
	case 1:
		if constexpr (is_int<T> && is_int<U>) {
			depth_kernel<T, U, 1, 0><<<grid, kThreads, 0, st>>>(L);
			return cudaGetLastError();
		}
		return cudaErrorInvalidValue;
	case 2:
		if constexpr (is_fp<U>) {
			depth_kernel<T, U, 2, 0><<<grid, kThreads, 0, st>>>(L);
			return cudaGetLastError();
		}
		return cudaErrorInvalidValue;
	case 3:
		if constexpr (is_int<U>) {
			if (L.dither == 1)
				depth_kernel<T, U, 3, 1><<<grid, kThreads, 0, st>>>(L);
			else if (L.dither == 2)
				depth_kernel<T, U, 3, 2><<<grid, kThreads, 0, st>>>(L);
			else
				depth_kernel<T, U, 3, 0><<<grid, kThreads, 0, st>>>(L);
			return cudaGetLastError();
		}
		return cudaErrorInvalidValue;
	default: return cudaErrorInvalidValue;
	}
}

template <class T>
cudaError_t launch_t(int out_type, int mode, const DepthLaunch &L, int grid, cudaStream_t st)
{
	switch (out_type) {
	case 0: return launch_tu<T, uint8_t>(mode, L, grid, st);
	case 1: return launch_tu<T, uint16_t>(mode, L, grid, st);
	case 2: return launch_tu<T, Half>(mode, L, grid, st);
	case 3: return launch_tu<T, float>(mode, L, grid, st);
	default: return cudaErrorInvalidValue;
	}
}

} // namespace

cudaError_t launch_depth(int in_type, int out_type, int mode, const DepthLaunch &L, cudaStream_t stream)
{
	if (L.width <= 0 || L.height <= 0)
		return cudaSuccess;
	static int sms = 0;
	if (!sms) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (sms < 1)
			sms = 1;
	}
	const long long runs = static_cast<long long>((L.width + kRun - 1) / kRun) * L.height;
	const int grid = static_cast<int>(std::min<long long>((runs + kThreads - 1) / kThreads, static_cast<long long>(sms) * 8));
	switch (in_type) {
	case 0: return launch_t<uint8_t>(out_type, mode, L, grid, stream);
	case 1: return launch_t<uint16_t>(out_type, mode, L, grid, stream);
	case 2: return launch_t<Half>(out_type, mode, L, grid, stream);
	case 3: return launch_t<float>(out_type, mode, L, grid, stream);
	default: return cudaErrorInvalidValue;
	}
}

} // namespace zg
