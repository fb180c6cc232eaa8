// Single-pass resize kernels: one horizontal or vertical banded pass over a
// whole plane, for any tap count. These are the general path (and the
// building block of two-pass conversions whose intermediate lives in HBM).
//
// Arithmetic, per output sample, is exactly zimg's C path
// (src/zimg/resize/resize_impl.cpp:31-114):
//   u16: int32 sum of int16 tap * (x - 32768), then ((sum + 8192) >> 14) + 32768
//        clamped to [0, 2^depth - 1]  -> bit-exact;
//   f32: taps applied in order k = 0..width-1 with a fused multiply-add per tap.
#include "kernels.h"

#include <algorithm>

namespace zg {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ uint16_t pack_u16(uint32_t acc, int32_t pixel_max)
{
	int32_t x = (static_cast<int32_t>(acc + 8192u) >> 14) + 32768;
	x = min(max(x, 0), pixel_max);
	return static_cast<uint16_t>(x);
}

// ---------------------------------------------------------------- vertical --
// Thread = VEC adjacent columns; block = kThreads * VEC columns x `rows_per_block`
// output rows. Every load of a row segment is coalesced across the warp.
template <int VEC>
__global__ void __launch_bounds__(kThreads)
v_u16_kernel(PassTables t, int32_t pixel_max, unsigned plane_w, const uint8_t *__restrict__ src, ptrdiff_t ss,
             uint8_t *__restrict__ dst, ptrdiff_t ds, unsigned rows_per_block)
{
	const unsigned j0 = (blockIdx.x * kThreads + threadIdx.x) * VEC;
	if (j0 >= plane_w)
		return;
	const bool full = j0 + VEC <= plane_w;
	const unsigned i0 = blockIdx.y * rows_per_block;
	const unsigned i1 = min(i0 + rows_per_block, t.rows);

	for (unsigned i = i0; i < i1; ++i) {
		const unsigned top = __ldg(t.left + i);
		const int16_t *c = t.i16 + static_cast<size_t>(i) * t.width;
		uint32_t acc[VEC];
		const uint32_t b = static_cast<uint32_t>(__ldg(t.bias + i));
#pragma unroll
		for (int v = 0; v < VEC; ++v)
			acc[v] = b;

		const uint8_t *row = src + static_cast<ptrdiff_t>(top) * ss + static_cast<size_t>(j0) * 2;
		for (unsigned k = 0; k < t.width; ++k, row += ss) {
			const int32_t ck = __ldg(c + k);
			if (VEC == 8 && full) {
				uint4 q = __ldg(reinterpret_cast<const uint4 *>(row));
				const uint32_t w[4] = { q.x, q.y, q.z, q.w };
#pragma unroll
				for (int v = 0; v < 4; ++v) {
					acc[2 * v] += static_cast<uint32_t>(ck * static_cast<int32_t>(w[v] & 0xFFFFu));
					acc[2 * v + 1] += static_cast<uint32_t>(ck * static_cast<int32_t>(w[v] >> 16));
				}
			} else {
				const uint16_t *r16 = reinterpret_cast<const uint16_t *>(row);
#pragma unroll
				for (int v = 0; v < VEC; ++v)
					if (full || j0 + v < plane_w)
						acc[v] += static_cast<uint32_t>(ck * static_cast<int32_t>(__ldg(r16 + v)));
			}
		}

		uint16_t *out = reinterpret_cast<uint16_t *>(dst + static_cast<ptrdiff_t>(i) * ds) + j0;
		if (VEC == 8 && full) {
			uint32_t w[4];
#pragma unroll
			for (int v = 0; v < 4; ++v)
				w[v] = pack_u16(acc[2 * v], pixel_max) | (static_cast<uint32_t>(pack_u16(acc[2 * v + 1], pixel_max)) << 16);
			*reinterpret_cast<uint4 *>(out) = make_uint4(w[0], w[1], w[2], w[3]);
		} else {
#pragma unroll
			for (int v = 0; v < VEC; ++v)
				if (full || j0 + v < plane_w)
					out[v] = pack_u16(acc[v], pixel_max);
		}
	}
}

template <int VEC>
__global__ void __launch_bounds__(kThreads)
v_f32_kernel(PassTables t, unsigned plane_w, const uint8_t *__restrict__ src, ptrdiff_t ss,
             uint8_t *__restrict__ dst, ptrdiff_t ds, unsigned rows_per_block)
{
	const unsigned j0 = (blockIdx.x * kThreads + threadIdx.x) * VEC;
	if (j0 >= plane_w)
		return;
	const bool full = j0 + VEC <= plane_w;
	const unsigned i0 = blockIdx.y * rows_per_block;
	const unsigned i1 = min(i0 + rows_per_block, t.rows);

	for (unsigned i = i0; i < i1; ++i) {
		const unsigned top = __ldg(t.left + i);
		const float *c = t.f32 + static_cast<size_t>(i) * t.width;
		float acc[VEC];
#pragma unroll
		for (int v = 0; v < VEC; ++v)
			acc[v] = 0.0f;

		const uint8_t *row = src + static_cast<ptrdiff_t>(top) * ss + static_cast<size_t>(j0) * 4;
		for (unsigned k = 0; k < t.width; ++k, row += ss) {
			const float ck = __ldg(c + k);
			if (VEC == 4 && full) {
				float4 q = __ldg(reinterpret_cast<const float4 *>(row));
				acc[0] = __fmaf_rn(ck, q.x, acc[0]);
				acc[1] = __fmaf_rn(ck, q.y, acc[1]);
				acc[2] = __fmaf_rn(ck, q.z, acc[2]);
				acc[3] = __fmaf_rn(ck, q.w, acc[3]);
			} else {
				const float *rf = reinterpret_cast<const float *>(row);
#pragma unroll
				for (int v = 0; v < VEC; ++v)
					if (full || j0 + v < plane_w)
						acc[v] = __fmaf_rn(ck, __ldg(rf + v), acc[v]);
			}
		}

		float *out = reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(i) * ds) + j0;
		if (VEC == 4 && full) {
			*reinterpret_cast<float4 *>(out) = make_float4(acc[0], acc[1], acc[2], acc[3]);
		} else {
#pragma unroll
			for (int v = 0; v < VEC; ++v)
				if (full || j0 + v < plane_w)
					out[v] = acc[v];
		}
	}
}

// -------------------------------------------------------------- horizontal --
// Thread = one output column for `rows_per_block` lines; its taps stay in L1.
__global__ void __launch_bounds__(kThreads)
h_u16_kernel(PassTables t, int32_t pixel_max, unsigned lines, const uint8_t *__restrict__ src, ptrdiff_t ss,
             uint8_t *__restrict__ dst, ptrdiff_t ds, unsigned rows_per_block)
{
	const unsigned j = blockIdx.x * kThreads + threadIdx.x;
	if (j >= t.rows)
		return;
	const unsigned l = __ldg(t.left + j);
	const int16_t *c = t.i16 + static_cast<size_t>(j) * t.width;
	const uint32_t b = static_cast<uint32_t>(__ldg(t.bias + j));
	const unsigned r0 = blockIdx.y * rows_per_block;
	const unsigned r1 = min(r0 + rows_per_block, lines);
	for (unsigned r = r0; r < r1; ++r) {
		const uint16_t *s = reinterpret_cast<const uint16_t *>(src + static_cast<ptrdiff_t>(r) * ss) + l;
		uint32_t acc = b;
		for (unsigned k = 0; k < t.width; ++k)
			acc += static_cast<uint32_t>(static_cast<int32_t>(__ldg(c + k)) * static_cast<int32_t>(__ldg(s + k)));
		reinterpret_cast<uint16_t *>(dst + static_cast<ptrdiff_t>(r) * ds)[j] = pack_u16(acc, pixel_max);
	}
}

__global__ void __launch_bounds__(kThreads)
h_f32_kernel(PassTables t, unsigned lines, const uint8_t *__restrict__ src, ptrdiff_t ss,
             uint8_t *__restrict__ dst, ptrdiff_t ds, unsigned rows_per_block)
{
	const unsigned j = blockIdx.x * kThreads + threadIdx.x;
	if (j >= t.rows)
		return;
	const unsigned l = __ldg(t.left + j);
	const float *c = t.f32 + static_cast<size_t>(j) * t.width;
	const unsigned r0 = blockIdx.y * rows_per_block;
	const unsigned r1 = min(r0 + rows_per_block, lines);
	for (unsigned r = r0; r < r1; ++r) {
		const float *s = reinterpret_cast<const float *>(src + static_cast<ptrdiff_t>(r) * ss) + l;
		float acc = 0.0f;
		for (unsigned k = 0; k < t.width; ++k)
			acc = __fmaf_rn(__ldg(c + k), __ldg(s + k), acc);
		reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(r) * ds)[j] = acc;
	}
}

// ------------------------------------------------------ wide, CUDA cores --
// FP32 passes of kDenseTaps taps or more, on the dense groups of outputs
// (PassTables::dense). Each output's taps are applied in zimg's order, one
// fused multiply-add each; the block's zeros outside an output's band add
// 0 * x, which leaves an accumulator that started at +0 unchanged for finite
// samples (such an accumulator never becomes -0), so the results are those of
// the per-output kernels above.

constexpr unsigned kVRows = dense_rows(false);  // 8
constexpr unsigned kHRows = dense_rows(true);   // 4

// Vertical: thread = 4 adjacent columns (16-byte loads and stores, planes
// 16-byte aligned); block = kThreads * 4 columns x `groups_per_block` groups
// of 8 output rows. Per input line of a group's window: one load of the 4
// columns, the group's 8 taps of that line (two 16-byte loads, the same for
// every thread), 32 multiply-adds as 16 paired ones. A line is read once per
// group. Group size trades reads against work: a 16x downscale of 129 taps
// reads each line 1.9 times with 8 rows (1.4 with 16, 2.8 with 4) and its
// dense windows are 54 % taps (35 % with 16); 8 measured fastest (16 rows
// leave too few warps per plane).
__global__ void __launch_bounds__(kThreads)
v_f32_dense_kernel(PassTables t, unsigned plane_w, const uint8_t *__restrict__ src, ptrdiff_t ss,
                   uint8_t *__restrict__ dst, ptrdiff_t ds, unsigned groups_per_block)
{
	const unsigned j0 = (blockIdx.x * kThreads + threadIdx.x) * 4;
	if (j0 >= plane_w)
		return;
	const bool full = j0 + 4 <= plane_w;
	const unsigned ngroups = (t.rows + kVRows - 1) / kVRows;
	const unsigned g0 = blockIdx.y * groups_per_block;
	const unsigned g1 = min(g0 + groups_per_block, ngroups);
	for (unsigned g = g0; g < g1; ++g) {
		const unsigned base = __ldg(t.dbase + g), span = __ldg(t.dspan + g);
		const float4 *tap = reinterpret_cast<const float4 *>(t.dense) + static_cast<size_t>(g) * t.dstride * (kVRows / 4);
		float2 acc[kVRows][2];
#pragma unroll
		for (int r = 0; r < static_cast<int>(kVRows); ++r)
			acc[r][0] = acc[r][1] = make_float2(0.0f, 0.0f);
		const uint8_t *row = src + static_cast<ptrdiff_t>(base) * ss + static_cast<size_t>(j0) * 4;
#pragma unroll 2
		for (unsigned u = 0; u < span; ++u, row += ss) {
			float4 x;
			if (full) {
				x = __ldg(reinterpret_cast<const float4 *>(row));
			} else {
				const float *rf = reinterpret_cast<const float *>(row);
				x.x = __ldg(rf);
				x.y = j0 + 1 < plane_w ? __ldg(rf + 1) : 0.0f;
				x.z = j0 + 2 < plane_w ? __ldg(rf + 2) : 0.0f;
				x.w = j0 + 3 < plane_w ? __ldg(rf + 3) : 0.0f;
			}
			const float2 x01 = make_float2(x.x, x.y), x23 = make_float2(x.z, x.w);
#pragma unroll
			for (int q = 0; q < static_cast<int>(kVRows / 4); ++q) {
				const float4 c = __ldg(tap + u * (kVRows / 4) + q);
				const float cr[4] = { c.x, c.y, c.z, c.w };
#pragma unroll
				for (int e = 0; e < 4; ++e) {
					const float2 cc = make_float2(cr[e], cr[e]);
					acc[4 * q + e][0] = __ffma2_rn(cc, x01, acc[4 * q + e][0]);
					acc[4 * q + e][1] = __ffma2_rn(cc, x23, acc[4 * q + e][1]);
				}
			}
		}
#pragma unroll
		for (int r = 0; r < static_cast<int>(kVRows); ++r) {
			const unsigned i = g * kVRows + r;
			if (i >= t.rows)
				break;
			float *out = reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(i) * ds) + j0;
			if (full) {
				*reinterpret_cast<float4 *>(out) = make_float4(acc[r][0].x, acc[r][0].y, acc[r][1].x, acc[r][1].y);
			} else {
				const float v[4] = { acc[r][0].x, acc[r][0].y, acc[r][1].x, acc[r][1].y };
				for (int q = 0; q < 4 && j0 + q < plane_w; ++q)
					out[q] = v[q];
			}
		}
	}
}

// Horizontal: warp = one line x 32 consecutive groups of 4 outputs (lane =
// group). The warp first copies its groups' input window of the line into
// shared memory with coalesced loads (one pad word per 32, so that lanes
// whose windows start 2^n samples apart read different banks), then each
// lane runs its group: per input one sample from shared memory, the group's
// 4 taps (coalesced across the lanes: the table keeps 32 groups side by
// side), 4 multiply-adds. kHWarps lines per block.
constexpr int kHWarps = 4;

__host__ __device__ __forceinline__ unsigned hpad(unsigned i)
{
	return i + (i >> 5);
}

__global__ void __launch_bounds__(kHWarps * 32)
h_f32_dense_kernel(PassTables t, unsigned lines, const uint8_t *__restrict__ src, ptrdiff_t ss,
                   uint8_t *__restrict__ dst, ptrdiff_t ds)
{
	extern __shared__ float hwin[];
	const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const unsigned ngroups = (t.rows + kHRows - 1) / kHRows;
	const unsigned gw = blockIdx.x * 32;  // first group of the warp
	const unsigned r = blockIdx.y * kHWarps + warp;
	if (r >= lines)
		return;
	float *win = hwin + warp * hpad(t.dwin + 32);
	const unsigned glast = min(gw + 32, ngroups) - 1;
	const unsigned w0 = __ldg(t.dbase + gw);
	const unsigned wn = __ldg(t.dbase + glast) + __ldg(t.dspan + glast) - w0;
	const float *s = reinterpret_cast<const float *>(src + static_cast<ptrdiff_t>(r) * ss) + w0;
	for (unsigned i = lane; i < wn; i += 32)
		win[hpad(i)] = __ldg(s + i);
	__syncwarp();
	const unsigned g = gw + lane;
	if (g >= ngroups)
		return;
	const unsigned off = __ldg(t.dbase + g) - w0, span = __ldg(t.dspan + g);
	const float4 *tap = reinterpret_cast<const float4 *>(t.dense) + g;
	float2 acc01 = make_float2(0.0f, 0.0f), acc23 = make_float2(0.0f, 0.0f);
#pragma unroll 4
	for (unsigned u = 0; u < span; ++u) {
		const float4 c = __ldg(tap + static_cast<size_t>(u) * ngroups);
		const float x = win[hpad(off + u)];
		acc01 = __ffma2_rn(make_float2(c.x, c.y), make_float2(x, x), acc01);
		acc23 = __ffma2_rn(make_float2(c.z, c.w), make_float2(x, x), acc23);
	}
	float *out = reinterpret_cast<float *>(dst + static_cast<ptrdiff_t>(r) * ds) + g * kHRows;
	const float v[4] = { acc01.x, acc01.y, acc23.x, acc23.y };
#pragma unroll
	for (int q = 0; q < static_cast<int>(kHRows); ++q)
		if (g * kHRows + q < t.rows)
			out[q] = v[q];
}

bool aligned16(const void *p, ptrdiff_t stride)
{
	return (reinterpret_cast<uintptr_t>(p) % 16) == 0 && (stride % 16) == 0;
}

} // namespace


cudaError_t launch_pass(const PassLaunch &l, cudaStream_t stream)
{
	if (l.wide.frag && l.sample == Sample::F32)
		return launch_wide(l, stream);
	const uint8_t *src = static_cast<const uint8_t *>(l.src);
	uint8_t *dst = static_cast<uint8_t *>(l.dst);
	if (l.sample == Sample::F32 && l.t.dense) {
		if (l.horizontal) {
			// staged windows of 32 groups, up to 16 KB per warp
			const size_t win_bytes = static_cast<size_t>(hpad(l.t.dwin + 32)) * 4;
			if (win_bytes <= 16384) {
				const unsigned groups = (l.t.rows + kHRows - 1) / kHRows;
				dim3 grid((groups + 31) / 32, (l.lines + kHWarps - 1) / kHWarps);
				cudaError_t e = cudaFuncSetAttribute(h_f32_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
				                                     static_cast<int>(kHWarps * 16384 + 4096));
				if (e != cudaSuccess)
					return e;
				h_f32_dense_kernel<<<grid, kHWarps * 32, kHWarps * win_bytes, stream>>>(l.t, l.lines, src,
				                                                                      l.src_stride, dst, l.dst_stride);
				return cudaGetLastError();
			}
		} else if (aligned16(l.src, l.src_stride) && aligned16(l.dst, l.dst_stride)) {
			const unsigned groups = (l.t.rows + kVRows - 1) / kVRows;
			const unsigned col_blocks = (l.lines + kThreads * 4 - 1) / (kThreads * 4);
			dim3 grid(col_blocks, groups);
			v_f32_dense_kernel<<<grid, kThreads, 0, stream>>>(l.t, l.lines, src, l.src_stride, dst, l.dst_stride, 1);
			return cudaGetLastError();
		}
	}
	if (l.horizontal) {
		const unsigned rpb = 8;
		dim3 grid((l.t.rows + kThreads - 1) / kThreads, (l.lines + rpb - 1) / rpb);
		if (l.sample == Sample::U16)
			h_u16_kernel<<<grid, kThreads, 0, stream>>>(l.t, l.pixel_max, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
		else
			h_f32_kernel<<<grid, kThreads, 0, stream>>>(l.t, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
	} else {
		const unsigned rpb = 4;
		const bool vec = aligned16(l.src, l.src_stride) && aligned16(l.dst, l.dst_stride);
		if (l.sample == Sample::U16) {
			const int V = vec ? 8 : 1;
			dim3 grid((l.lines + kThreads * V - 1) / (kThreads * V), (l.t.rows + rpb - 1) / rpb);
			if (vec)
				v_u16_kernel<8><<<grid, kThreads, 0, stream>>>(l.t, l.pixel_max, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
			else
				v_u16_kernel<1><<<grid, kThreads, 0, stream>>>(l.t, l.pixel_max, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
		} else {
			const int V = vec ? 4 : 1;
			dim3 grid((l.lines + kThreads * V - 1) / (kThreads * V), (l.t.rows + rpb - 1) / rpb);
			if (vec)
				v_f32_kernel<4><<<grid, kThreads, 0, stream>>>(l.t, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
			else
				v_f32_kernel<1><<<grid, kThreads, 0, stream>>>(l.t, l.lines, src, l.src_stride, dst, l.dst_stride, rpb);
		}
	}
	return cudaGetLastError();
}

} // namespace zg
