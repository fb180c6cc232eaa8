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
