// Unresize passes on the GPU (zimg's unresize_impl.cpp:27-97, C path): per
// output sample a banded FP32 dot product with A''s row, then the forward
// substitution of the tridiagonal LU, then the back substitution; every
// product, sum and difference rounded on its own, as in zimg's C code.
//
// A pass is two launches. The dot products do not depend on the recurrence,
// so one thread per output sample computes them (k in zimg's order) into the
// pass's output plane. The substitutions are recurrences along the line
// (horizontal pass) or down the column (vertical pass): one thread each,
// rewriting the plane in place, with the next inputs loaded before the
// dependent steps so that memory latency overlaps the chain (down a column in
// groups of kAhead values; along lines a warp moves tiles of 32 lines x 32
// values through shared memory).
#include "unresize.h"

#include <algorithm>

namespace zg {

namespace {

constexpr int kThreads = 128;
constexpr int kAhead = 32;  // recurrence inputs loaded per group

// dst[line][j] = sum_k coef[j][k] * src[line][offset[j] + k]
__global__ void __launch_bounds__(kThreads)
unresize_dot_h(UnresizeTables t, unsigned lines, const char *__restrict__ src, ptrdiff_t ss, char *__restrict__ dst,
               ptrdiff_t ds)
{
	const unsigned j = blockIdx.x * kThreads + threadIdx.x;
	if (j >= t.orig)
		return;
	const float *cf = t.coef + static_cast<size_t>(j) * t.row_size;
	const unsigned off = __ldg(t.offset + j);
	for (unsigned line = blockIdx.y; line < lines; line += gridDim.y) {
		const float *x = reinterpret_cast<const float *>(src + static_cast<ptrdiff_t>(line) * ss) + off;
		float accum = 0.0f;
		for (unsigned k = 0; k < t.row_size; ++k)
			accum = __fadd_rn(accum, __fmul_rn(__ldg(cf + k), __ldg(x + k)));
		reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(line) * ds)[j] = accum;
	}
}

// dst[i][col] = sum_k coef[i][k] * src[offset[i] + k][col]
__global__ void __launch_bounds__(kThreads)
unresize_dot_v(UnresizeTables t, unsigned cols, const char *__restrict__ src, ptrdiff_t ss, char *__restrict__ dst,
               ptrdiff_t ds)
{
	const unsigned col = blockIdx.x * kThreads + threadIdx.x;
	if (col >= cols)
		return;
	for (unsigned i = blockIdx.y; i < t.orig; i += gridDim.y) {
		const float *cf = t.coef + static_cast<size_t>(i) * t.row_size;
		const char *x = src + static_cast<ptrdiff_t>(__ldg(t.offset + i)) * ss + static_cast<size_t>(col) * 4;
		float accum = 0.0f;
		for (unsigned k = 0; k < t.row_size; ++k)
			accum = __fadd_rn(accum, __fmul_rn(__ldg(cf + k),
			                                   __ldg(reinterpret_cast<const float *>(x + static_cast<ptrdiff_t>(k) * ss))));
		reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(i) * ds)[col] = accum;
	}
}

// The substitutions over n values at p, p + step, ... (step in floats):
// z_i = (a_i - c_i z_{i-1}) * l_i, then w_i = z_i - u_i w_{i+1}. Inputs go
// in groups of kAhead; group g + 1 is loaded before group g's steps run.
__device__ __forceinline__ void substitute(const UnresizeTables &t, float *p, ptrdiff_t step, unsigned n)
{
	auto at = [&](unsigned i) -> float & { return p[static_cast<ptrdiff_t>(i) * step]; };
	float z = 0.0f;
	const unsigned full = n / kAhead * kAhead;
	float cur[kAhead], nxt[kAhead];
	if (full) {
#pragma unroll
		for (int e = 0; e < kAhead; ++e)
			cur[e] = at(e);
	}
	for (unsigned i = 0; i < full; i += kAhead) {
		if (i + kAhead < full) {
#pragma unroll
			for (int e = 0; e < kAhead; ++e)
				nxt[e] = at(i + kAhead + e);
		}
#pragma unroll
		for (int e = 0; e < kAhead; ++e) {
			z = __fmul_rn(__fsub_rn(cur[e], __fmul_rn(__ldg(t.lu_c + i + e), z)), __ldg(t.lu_l + i + e));
			at(i + e) = z;
		}
#pragma unroll
		for (int e = 0; e < kAhead; ++e)
			cur[e] = nxt[e];
	}
	for (unsigned i = full; i < n; ++i) {
		z = __fmul_rn(__fsub_rn(at(i), __fmul_rn(__ldg(t.lu_c + i), z)), __ldg(t.lu_l + i));
		at(i) = z;
	}
	// back substitution from the last value: the partial group first
	float w = 0.0f;
	for (unsigned r = n; r > full; --r) {
		w = __fsub_rn(at(r - 1), __fmul_rn(__ldg(t.lu_u + r - 1), w));
		at(r - 1) = w;
	}
	if (full) {
#pragma unroll
		for (int e = 0; e < kAhead; ++e)
			cur[e] = at(full - 1 - e);
	}
	for (unsigned r = full; r != 0; r -= kAhead) {
		if (r > kAhead) {
#pragma unroll
			for (int e = 0; e < kAhead; ++e)
				nxt[e] = at(r - kAhead - 1 - e);
		}
#pragma unroll
		for (int e = 0; e < kAhead; ++e) {
			w = __fsub_rn(cur[e], __fmul_rn(__ldg(t.lu_u + r - 1 - e), w));
			at(r - 1 - e) = w;
		}
#pragma unroll
		for (int e = 0; e < kAhead; ++e)
			cur[e] = nxt[e];
	}
}

// Horizontal substitutions, one warp per 32 lines: a line's values are
// contiguous, so a thread per line would read 32 rows per warp load. The warp
// moves tiles of 32 lines x 32 values through shared memory instead (one
// 128-byte row per load instruction, the next two tiles in flight in
// registers), and each lane runs its own line's recurrence on the tile;
// the arithmetic and its order are those of substitute().
constexpr int kTile = 32;

struct HTile {
	float v[kTile];  // this lane's column of the tile: rows 0 .. 31
};

__device__ __forceinline__ void load_tile(HTile &r, const char *dst, ptrdiff_t ds, unsigned line0, unsigned lines,
                                          unsigned col0, unsigned n)
{
	const unsigned lane = threadIdx.x & 31, c = col0 + lane;
#pragma unroll
	for (int i = 0; i < kTile; ++i)
		r.v[i] = (line0 + i < lines && c < n)
		             ? reinterpret_cast<const float *>(dst + static_cast<ptrdiff_t>(line0 + i) * ds)[c]
		             : 0.0f;
}

__global__ void __launch_bounds__(32)
unresize_subst_h(UnresizeTables t, unsigned lines, char *__restrict__ dst, ptrdiff_t ds)
{
	__shared__ float tile[kTile][kTile + 1];
	const unsigned lane = threadIdx.x & 31, line0 = blockIdx.x * kTile;
	const unsigned n = t.orig, tiles = (n + kTile - 1) / kTile;
	const bool mine = line0 + lane < lines;
	// one pass over the tiles, forward (z) or backward (w); row `lane` of a
	// tile is this lane's line
	auto pass = [&](bool forward) {
		HTile a, b;
		float carry = 0.0f;
		const unsigned first = forward ? 0 : tiles - 1;
		load_tile(a, dst, ds, line0, lines, first * kTile, n);
		if (tiles > 1)
			load_tile(b, dst, ds, line0, lines, (forward ? first + 1 : first - 1) * kTile, n);
		for (unsigned k = 0; k < tiles; ++k) {
			const unsigned j = forward ? k : tiles - 1 - k;
			const unsigned col0 = j * kTile, cnt = min(static_cast<unsigned>(kTile), n - col0);
#pragma unroll
			for (int i = 0; i < kTile; ++i)
				tile[i][lane] = a.v[i];
			a = b;
			if (k + 2 < tiles)
				load_tile(b, dst, ds, line0, lines, (forward ? j + 2 : j - 2) * kTile, n);
			__syncwarp();
			if (mine) {
				// whole tiles unrolled, so that the coefficient loads run ahead of the chain
				if (forward && cnt == kTile) {
#pragma unroll
					for (int c = 0; c < kTile; ++c) {
						carry = __fmul_rn(__fsub_rn(tile[lane][c], __fmul_rn(__ldg(t.lu_c + col0 + c), carry)),
						                  __ldg(t.lu_l + col0 + c));
						tile[lane][c] = carry;
					}
				} else if (forward) {
					for (unsigned c = 0; c < cnt; ++c) {
						carry = __fmul_rn(__fsub_rn(tile[lane][c], __fmul_rn(__ldg(t.lu_c + col0 + c), carry)),
						                  __ldg(t.lu_l + col0 + c));
						tile[lane][c] = carry;
					}
				} else if (cnt == kTile) {
#pragma unroll
					for (int c = kTile - 1; c >= 0; --c) {
						carry = __fsub_rn(tile[lane][c], __fmul_rn(__ldg(t.lu_u + col0 + c), carry));
						tile[lane][c] = carry;
					}
				} else {
					for (unsigned c = cnt; c-- > 0;) {
						carry = __fsub_rn(tile[lane][c], __fmul_rn(__ldg(t.lu_u + col0 + c), carry));
						tile[lane][c] = carry;
					}
				}
			}
			__syncwarp();
			const unsigned cc = col0 + lane;
			if (cc < n) {
#pragma unroll
				for (int i = 0; i < kTile; ++i)
					if (line0 + i < lines)
						reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(line0 + i) * ds)[cc] = tile[i][lane];
			}
			__syncwarp();
		}
	};
	pass(true);
	pass(false);
}

__global__ void __launch_bounds__(kThreads)
unresize_subst_v(UnresizeTables t, unsigned cols, char *__restrict__ dst, ptrdiff_t ds)
{
	const unsigned col = blockIdx.x * kThreads + threadIdx.x;
	if (col < cols)
		substitute(t, reinterpret_cast<float *>(dst) + col, ds / 4, t.orig);
}

} // namespace

cudaError_t launch_unresize(const UnresizeTables &t, bool horizontal, unsigned lines_or_cols, const void *src,
                            ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride, cudaStream_t stream)
{
	if (!lines_or_cols || !t.orig)
		return cudaSuccess;
	const unsigned n = lines_or_cols;
	const char *s = static_cast<const char *>(src);
	char *d = static_cast<char *>(dst);
	constexpr unsigned kGridY = 65535;  // CUDA's limit; the kernels stride over the rest
	if (horizontal) {
		unresize_dot_h<<<dim3((t.orig + kThreads - 1) / kThreads, std::min(n, kGridY)), kThreads, 0, stream>>>(
			t, n, s, src_stride, d, dst_stride);
		unresize_subst_h<<<(n + kTile - 1) / kTile, 32, 0, stream>>>(t, n, d, dst_stride);
	} else {
		unresize_dot_v<<<dim3((n + kThreads - 1) / kThreads, std::min(t.orig, kGridY)), kThreads, 0, stream>>>(
			t, n, s, src_stride, d, dst_stride);
		unresize_subst_v<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(t, n, d, dst_stride);
	}
	return cudaGetLastError();
}

} // namespace zg
