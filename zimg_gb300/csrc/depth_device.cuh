// Device helpers shared by the depth kernels (depth_kernel.cu, ed_kernel.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

namespace zg {

// HALF samples: IEEE binary16 bits, a type of its own so that templates do
// not take them for WORD.
struct Half {
	uint16_t bits;
};

// binary16 -> binary32, exact; NaNs stay NaN with the quiet bit set.
__device__ __forceinline__ float half_bits_to_float(uint32_t h)
{
	const uint32_t sign = (h & 0x8000u) << 16;
	const uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
	if (e == 0x1Fu)
		return __uint_as_float(sign | 0x7F800000u | (m ? ((m << 13) | 0x00400000u) : 0u));
	if (e == 0) {
		// zero or subnormal: m * 2^-24, exact in binary32
		const float v = __fmul_rn(static_cast<float>(m), 5.9604644775390625e-8f);
		return __uint_as_float(__float_as_uint(v) | sign);
	}
	return __uint_as_float(sign | ((e + 112u) << 23) | (m << 13));
}

// one sample as float: integers exactly, HALF widened exactly
template <class T>
__device__ __forceinline__ float sample_to_float(T v)
{
	if constexpr (std::is_same_v<T, Half>)
		return half_bits_to_float(v.bits);
	else
		return static_cast<float>(v);
}

} // namespace zg
