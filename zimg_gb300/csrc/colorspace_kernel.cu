// Colorspace conversion of three FLOAT planes (zimg's ColorspaceConversionImpl,
// src/zimg/colorspace/colorspace.cpp:16-78, operations of
// operation_impl.cpp:21-258): every operation of the plan applied to a pixel
// in registers, one pass over the planes. HBM-bound for matrix-only plans
// (12 bytes read and 12 written per pixel); transfer functions add a few
// dozen instructions per channel. Each thread converts runs of 4 pixels of a
// line (16-byte vectors where all planes allow). Every product, sum and
// quotient is written with the separately rounding CS_* forms, as zimg's C
// code rounds them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>

#include "colorspace_plan.h"
#include "colorspace_tf.cuh"

namespace zg {
namespace csp {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void apply_op(const Op &o, float &a, float &b, float &c)
{
	switch (o.kind) {
	case OP_MATRIX: {
		const float x = CS_ADD(CS_ADD(CS_MUL(o.m[0][0], a), CS_MUL(o.m[0][1], b)), CS_MUL(o.m[0][2], c));
		const float y = CS_ADD(CS_ADD(CS_MUL(o.m[1][0], a), CS_MUL(o.m[1][1], b)), CS_MUL(o.m[1][2], c));
		const float z = CS_ADD(CS_ADD(CS_MUL(o.m[2][0], a), CS_MUL(o.m[2][1], b)), CS_MUL(o.m[2][2], c));
		a = x;
		b = y;
		c = z;
		break;
	}
	case OP_GAMMA:
		a = CS_MUL(o.post, apply_tf(o.f, CS_MUL(a, o.pre)));
		b = CS_MUL(o.post, apply_tf(o.f, CS_MUL(b, o.pre)));
		c = CS_MUL(o.post, apply_tf(o.f, CS_MUL(c, o.pre)));
		break;
	case OP_HLG: {
		// display-referred HLG: system gamma 1.2 on the luma (operation_impl.cpp:76-114)
		const float gamma = 1.2f;
		const float r = CS_MUL(a, o.scale), g = CS_MUL(b, o.scale), bb = CS_MUL(c, o.scale);
		float yd = CS_ADD(CS_ADD(CS_MUL(o.kr, r), CS_MUL(o.kg, g)), CS_MUL(o.kb, bb));
		yd = yd < FLT_MIN ? FLT_MIN : yd;
		const float ys_inv = powf(yd, (1.0f - gamma) / gamma);
		a = hlg_oetf(CS_MUL(r, ys_inv));
		b = hlg_oetf(CS_MUL(g, ys_inv));
		c = hlg_oetf(CS_MUL(bb, ys_inv));
		break;
	}
	case OP_HLG_INV: {
		const float gamma = 1.2f;
		float r = hlg_inv_oetf(a), g = hlg_inv_oetf(b), bb = hlg_inv_oetf(c);
		float ys = CS_ADD(CS_ADD(CS_MUL(o.kr, r), CS_MUL(o.kg, g)), CS_MUL(o.kb, bb));
		ys = ys < FLT_MIN ? FLT_MIN : ys;
		ys = powf(ys, gamma - 1.0f);
		r = CS_MUL(r, ys);
		g = CS_MUL(g, ys);
		bb = CS_MUL(bb, ys);
		a = CS_MUL(r, o.scale);
		b = CS_MUL(g, o.scale);
		c = CS_MUL(bb, o.scale);
		break;
	}
	case OP_CL_TO_RGB: {
		// BT.2020 constant luminance to linear RGB (operation_impl.cpp:156-206)
		const float y = a, u = b, v = c;
		const float bmy = u < 0 ? CS_MUL(CS_MUL(u, 2.0f), o.nb) : CS_MUL(CS_MUL(u, 2.0f), o.pb);
		const float rmy = v < 0 ? CS_MUL(CS_MUL(v, 2.0f), o.nr) : CS_MUL(CS_MUL(v, 2.0f), o.pr);
		const float bl = apply_tf(o.f, CS_ADD(bmy, y)), rl = apply_tf(o.f, CS_ADD(rmy, y)), yl = apply_tf(o.f, y);
		const float g = CS_DIV(CS_SUB(CS_SUB(yl, CS_MUL(o.kr, rl)), CS_MUL(o.kb, bl)), o.kg);
		a = CS_MUL(rl, o.scale);
		b = CS_MUL(g, o.scale);
		c = CS_MUL(bl, o.scale);
		break;
	}
	case OP_CL_TO_YUV: {
		// linear RGB to BT.2020 constant luminance (operation_impl.cpp:209-258)
		float r = CS_MUL(a, o.scale), g = CS_MUL(b, o.scale), bb = CS_MUL(c, o.scale);
		const float y = apply_tf(o.f, CS_ADD(CS_ADD(CS_MUL(o.kr, r), CS_MUL(o.kg, g)), CS_MUL(o.kb, bb)));
		bb = apply_tf(o.f, bb);
		r = apply_tf(o.f, r);
		const float bmy = CS_SUB(bb, y), rmy = CS_SUB(r, y);
		const float u = bmy < 0.0f ? CS_DIV(bmy, CS_MUL(2.0f, o.nb)) : CS_DIV(bmy, CS_MUL(2.0f, o.pb));
		const float v = rmy < 0.0f ? CS_DIV(rmy, CS_MUL(2.0f, o.nr)) : CS_DIV(rmy, CS_MUL(2.0f, o.pr));
		a = y;
		b = u;
		c = v;
		break;
	}
	default: break;
	}
}

__global__ void __launch_bounds__(kThreads) colorspace_kernel(const __grid_constant__ Launch L)
{
	const int quads = (L.width + 3) / 4;
	const long long total = static_cast<long long>(quads) * L.height;
	for (long long u = static_cast<long long>(blockIdx.x) * kThreads + threadIdx.x; u < total;
	     u += static_cast<long long>(gridDim.x) * kThreads) {
		const int i = static_cast<int>(u / quads);
		const int j0 = static_cast<int>(u - static_cast<long long>(i) * quads) * 4;
		const int n = min(4, L.width - j0);
		const float *s[3];
		float *d[3];
#pragma unroll
		for (int p = 0; p < 3; ++p) {
			s[p] = reinterpret_cast<const float *>(static_cast<const char *>(L.src[p]) +
			                                       static_cast<ptrdiff_t>(i) * L.src_stride[p]) + j0;
			d[p] = reinterpret_cast<float *>(static_cast<char *>(L.dst[p]) + static_cast<ptrdiff_t>(i) * L.dst_stride[p]) +
			       j0;
		}
		float x[3][4];
		if (L.vec && n == 4) {
#pragma unroll
			for (int p = 0; p < 3; ++p) {
				const float4 v = *reinterpret_cast<const float4 *>(s[p]);
				x[p][0] = v.x;
				x[p][1] = v.y;
				x[p][2] = v.z;
				x[p][3] = v.w;
			}
		} else {
#pragma unroll
			for (int e = 0; e < 4; ++e)
#pragma unroll
				for (int p = 0; p < 3; ++p)
					x[p][e] = e < n ? s[p][e] : 0.0f;
		}
		for (int k = 0; k < L.plan.num_ops; ++k) {
			const Op &o = L.plan.ops[k];
#pragma unroll
			for (int e = 0; e < 4; ++e)
				apply_op(o, x[0][e], x[1][e], x[2][e]);
		}
		if (L.vec && n == 4) {
#pragma unroll
			for (int p = 0; p < 3; ++p)
				*reinterpret_cast<float4 *>(d[p]) = make_float4(x[p][0], x[p][1], x[p][2], x[p][3]);
		} else {
			for (int e = 0; e < n; ++e)
#pragma unroll
				for (int p = 0; p < 3; ++p)
					d[p][e] = x[p][e];
		}
	}
}

} // namespace

cudaError_t launch_colorspace(const Launch &L, cudaStream_t stream)
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
	const long long units = static_cast<long long>((L.width + 3) / 4) * L.height;
	const int grid = static_cast<int>(std::min<long long>((units + kThreads - 1) / kThreads, static_cast<long long>(sms) * 8));
	colorspace_kernel<<<grid, kThreads, 0, stream>>>(L);
	return cudaGetLastError();
}

} // namespace csp
} // namespace zg
