// Transfer functions of zimg's colorspace conversion (src/zimg/colorspace/
// gamma.cpp:12-343) for host and device: the constants are the published
// ones of BT.709, SMPTE 240M, IEC 61966-2-1 (sRGB, with zimg's continuity-
// adjusted pair), SMPTE ST 2084, ARIB STD-B67 and ST 428-1; the piecewise
// forms and their order of operations follow zimg's C code. On the host the
// library functions are the C library's, as zimg's; on the device CUDA's
// (powf, logf, log10f, expf within their documented error bounds, sqrtf
// correctly rounded). Every product, sum and quotient of these functions is
// written with CS_MUL / CS_ADD / CS_SUB / CS_DIV, which round on their own
// on the device (never contracted into a fused multiply-add), as zimg's C
// code rounds them; the library functions are free to contract inside.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace zg {
namespace csp {

#if defined(__CUDA_ARCH__)
#define ZG_CSP_FN __device__ __forceinline__
#define CS_MUL(a, b) __fmul_rn((a), (b))
#define CS_ADD(a, b) __fadd_rn((a), (b))
#define CS_SUB(a, b) __fsub_rn((a), (b))
#define CS_DIV(a, b) __fdiv_rn((a), (b))
#else
#define ZG_CSP_FN inline
#define CS_MUL(a, b) ((a) * (b))
#define CS_ADD(a, b) ((a) + (b))
#define CS_SUB(a, b) ((a) - (b))
#define CS_DIV(a, b) ((a) / (b))
#endif

constexpr float k709Alpha = 1.09929682680944f, k709Beta = 0.018053968510807f;
constexpr float k240Alpha = 1.111572195921731f, k240Beta = 0.022821585529445f;
constexpr float kSrgbAlpha = 1.055010718947587f, kSrgbBeta = 0.003041282560128f;
constexpr float kPqM1 = 0.1593017578125f, kPqM2 = 78.84375f;
constexpr float kPqC1 = 0.8359375f, kPqC2 = 18.8515625f, kPqC3 = 18.6875f;
constexpr float kHlgA = 0.17883277f, kHlgB = 0.28466892f, kHlgC = 0.55991073f;
constexpr float kPqOotfScale = 59.49080238715383f;  // BT.2390-2 5.3.1

// Transfer function ids (host plan -> device switch).
enum Tf : int {
	TF_709_OETF, TF_709_INV_OETF, TF_LOG100, TF_LOG100_INV, TF_LOG316, TF_LOG316_INV, TF_470M, TF_470M_INV,
	TF_470BG, TF_470BG_INV, TF_240M_OETF, TF_240M_INV_OETF, TF_XVYCC_OETF, TF_XVYCC_INV_OETF, TF_1361_OETF,
	TF_1361_INV_OETF, TF_HLG_OETF, TF_HLG_INV_OETF, TF_1886, TF_1886_INV, TF_SRGB, TF_SRGB_INV, TF_1361_EOTF,
	TF_1361_INV_EOTF, TF_XVYCC_EOTF, TF_XVYCC_INV_EOTF, TF_PQ_EOTF, TF_PQ_INV_EOTF, TF_428, TF_428_INV,
	TF_HLG_EOTF, TF_HLG_INV_EOTF, TF_PQ_OETF, TF_PQ_INV_OETF, TF_COUNT
};

// std::max(x, 0.0f): a NaN passes through
ZG_CSP_FN float max0(float x) { return x < 0.0f ? 0.0f : x; }

ZG_CSP_FN float pow_(float x, float y) { return powf(x, y); }
ZG_CSP_FN float log10_(float x) { return log10f(x); }
ZG_CSP_FN float log_(float x) { return logf(x); }
ZG_CSP_FN float exp_(float x) { return expf(x); }
ZG_CSP_FN float sqrt_(float x) { return sqrtf(x); }

// |x| and copysign on the bits
ZG_CSP_FN float abs_bits(float x)
{
	uint32_t u;
	memcpy(&u, &x, 4);
	u &= 0x7FFFFFFFu;
	memcpy(&x, &u, 4);
	return x;
}
ZG_CSP_FN float copysign_bits(float mag, float sgn)
{
	uint32_t a, b;
	memcpy(&a, &mag, 4);
	memcpy(&b, &sgn, 4);
	a = (a & 0x7FFFFFFFu) | (b & 0x80000000u);
	memcpy(&mag, &a, 4);
	return mag;
}

ZG_CSP_FN float bt709_oetf(float x)
{
	x = max0(x);
	return x < k709Beta ? CS_MUL(x, 4.5f) : CS_SUB(CS_MUL(k709Alpha, pow_(x, 0.45f)), k709Alpha - 1.0f);
}
ZG_CSP_FN float bt709_inv_oetf(float x)
{
	x = max0(x);
	return x < 4.5f * k709Beta ? CS_DIV(x, 4.5f) : pow_(CS_DIV(CS_ADD(x, k709Alpha - 1.0f), k709Alpha), 1.0f / 0.45f);
}
ZG_CSP_FN float bt1886(float x) { return x < 0.0f ? 0.0f : pow_(x, 2.4f); }
ZG_CSP_FN float bt1886_inv(float x) { return x < 0.0f ? 0.0f : pow_(x, 1.0f / 2.4f); }
ZG_CSP_FN float bt1361_oetf(float x) { return x >= 0.0f ? bt709_oetf(x) : CS_DIV(-bt709_oetf(CS_MUL(-x, 4.0f)), 4.0f); }
ZG_CSP_FN float bt1361_inv_oetf(float x) { return x >= 0.0f ? bt709_inv_oetf(x) : CS_DIV(-bt709_inv_oetf(CS_MUL(-x, 4.0f)), 4.0f); }
ZG_CSP_FN float xvycc_oetf(float x) { return copysign_bits(bt709_oetf(abs_bits(x)), x); }
ZG_CSP_FN float xvycc_inv_oetf(float x) { return copysign_bits(bt709_inv_oetf(abs_bits(x)), x); }
ZG_CSP_FN float hlg_oetf(float x)
{
	x = max0(x);
	return x <= (1.0f / 12.0f) ? sqrt_(CS_MUL(3.0f, x)) : CS_ADD(CS_MUL(kHlgA, log_(CS_SUB(CS_MUL(12.0f, x), kHlgB))), kHlgC);
}
ZG_CSP_FN float hlg_inv_oetf(float x)
{
	x = max0(x);
	return x <= 0.5f ? CS_MUL(CS_MUL(x, x), 1.0f / 3.0f) : CS_DIV(CS_ADD(exp_(CS_DIV(CS_SUB(x, kHlgC), kHlgA)), kHlgB), 12.0f);
}
ZG_CSP_FN float pq_eotf(float x)
{
	if (!(x > 0.0f))
		return 0.0f;
	const float xp = pow_(x, 1.0f / kPqM2);
	float num = CS_SUB(xp, kPqC1), den = CS_SUB(kPqC2, CS_MUL(kPqC3, xp));
	num = max0(num);
	den = den < FLT_MIN ? FLT_MIN : den;
	return pow_(CS_DIV(num, den), 1.0f / kPqM1);
}
ZG_CSP_FN float pq_inv_eotf(float x)
{
	if (!(x > 0.0f))
		return 0.0f;
	const float xp = pow_(x, kPqM1);
	const float num = CS_ADD(kPqC1 - 1.0f, CS_MUL(kPqC2 - kPqC3, xp));
	const float den = CS_ADD(1.0f, CS_MUL(kPqC3, xp));
	return pow_(CS_ADD(1.0f, CS_DIV(num, den)), kPqM2);
}

// One transfer function by id.
ZG_CSP_FN float apply_tf(int id, float x)
{
	switch (id) {
	case TF_709_OETF: return bt709_oetf(x);
	case TF_709_INV_OETF: return bt709_inv_oetf(x);
	case TF_LOG100: return x <= 0.01f ? 0.0f : CS_ADD(1.0f, CS_DIV(log10_(x), 2.0f));
	case TF_LOG100_INV: return x <= 0.0f ? 0.01f : pow_(10.0f, CS_MUL(2.0f, CS_SUB(x, 1.0f)));
	case TF_LOG316: return x <= 0.00316227766f ? 0.0f : CS_ADD(1.0f, CS_DIV(log10_(x), 2.5f));
	case TF_LOG316_INV: return x <= 0.0f ? 0.00316227766f : pow_(10.0f, CS_MUL(2.5f, CS_SUB(x, 1.0f)));
	case TF_470M: return x < 0.0f ? 0.0f : pow_(x, 2.2f);
	case TF_470M_INV: return x < 0.0f ? 0.0f : pow_(x, 1.0f / 2.2f);
	case TF_470BG: return x < 0.0f ? 0.0f : pow_(x, 2.8f);
	case TF_470BG_INV: return x < 0.0f ? 0.0f : pow_(x, 1.0f / 2.8f);
	case TF_240M_OETF: {
		x = max0(x);
		return x < 4.0f * k240Beta ? CS_DIV(x, 4.0f) : pow_(CS_DIV(CS_ADD(x, k240Alpha - 1.0f), k240Alpha), 1.0f / 0.45f);
	}
	case TF_240M_INV_OETF: {
		x = max0(x);
		return x < k240Beta ? CS_MUL(x, 4.0f) : CS_SUB(CS_MUL(k240Alpha, pow_(x, 0.45f)), k240Alpha - 1.0f);
	}
	case TF_XVYCC_OETF: return xvycc_oetf(x);
	case TF_XVYCC_INV_OETF: return xvycc_inv_oetf(x);
	case TF_1361_OETF: return bt1361_oetf(x);
	case TF_1361_INV_OETF: return bt1361_inv_oetf(x);
	case TF_HLG_OETF: return hlg_oetf(x);
	case TF_HLG_INV_OETF: return hlg_inv_oetf(x);
	case TF_1886: return bt1886(x);
	case TF_1886_INV: return bt1886_inv(x);
	case TF_SRGB: {
		x = max0(x);
		return x < 12.92f * kSrgbBeta ? CS_DIV(x, 12.92f) : pow_(CS_DIV(CS_ADD(x, kSrgbAlpha - 1.0f), kSrgbAlpha), 2.4f);
	}
	case TF_SRGB_INV: {
		x = max0(x);
		return x < kSrgbBeta ? CS_MUL(x, 12.92f) : CS_SUB(CS_MUL(kSrgbAlpha, pow_(x, 1.0f / 2.4f)), kSrgbAlpha - 1.0f);
	}
	case TF_1361_EOTF: return (x < 0.0f || x > 1.0f) ? bt1361_inv_oetf(x) : bt1886(x);
	case TF_1361_INV_EOTF: return (x < 0.0f || x > 1.0f) ? bt1361_oetf(x) : bt1886_inv(x);
	case TF_XVYCC_EOTF: return (x < 0.0f || x > 1.0f) ? xvycc_inv_oetf(x) : bt1886(x);
	case TF_XVYCC_INV_EOTF: return (x < 0.0f || x > 1.0f) ? xvycc_oetf(x) : bt1886_inv(x);
	case TF_PQ_EOTF: return pq_eotf(x);
	case TF_PQ_INV_EOTF: return pq_inv_eotf(x);
	case TF_428: return x < 0.0f ? 0.0f : CS_MUL(52.37f / 48.0f, pow_(x, 2.6f));
	case TF_428_INV: return x < 0.0f ? 0.0f : pow_(CS_MUL(x, 48.0f / 52.37f), 1.0f / 2.6f);
	case TF_HLG_EOTF: {
		// BT.2100 OOTF approximated per channel (gamma.cpp:316-320)
		const float l = hlg_inv_oetf(x);
		return l < 0.0f ? l : pow_(l, 1.2f);
	}
	case TF_HLG_INV_EOTF: return hlg_oetf(x < 0.0f ? x : pow_(x, 1.0f / 1.2f));
	case TF_PQ_OETF: return pq_inv_eotf(CS_DIV(bt1886(bt709_oetf(CS_MUL(x, kPqOotfScale))), 100.0f));
	case TF_PQ_INV_OETF: return CS_DIV(bt709_inv_oetf(bt1886_inv(CS_MUL(pq_eotf(x), 100.0f))), kPqOotfScale);
	default: return x;
	}
}

#undef ZG_CSP_FN

} // namespace csp
} // namespace zg
