// zimg's simple graph filters (src/zimg/graph/simple_filters.cpp): straight-
// alpha premultiply and unpremultiply of FLOAT planes (PremultiplyFilter /
// UnpremultiplyFilter, :69-110), one launch for up to three colour planes
// against one alpha plane, and a plane filled with one value
// (ValueInitializeFilter, :20-66). HBM-bound: each thread handles four
// samples of one line per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "alpha.h"

namespace zg {

namespace {

constexpr int kThreads = 256;

template <bool INVERSE>
__global__ void __launch_bounds__(kThreads) alpha_kernel(AlphaLaunch L)
{
	const int quads = (L.width + 3) / 4;
	const long long per_plane = static_cast<long long>(quads) * L.height;
	const long long total = per_plane * L.num_planes;
	for (long long u = static_cast<long long>(blockIdx.x) * kThreads + threadIdx.x; u < total;
	     u += static_cast<long long>(gridDim.x) * kThreads) {
		const int p = static_cast<int>(u / per_plane);
		const long long r = u - p * per_plane;
		const int i = static_cast<int>(r / quads);
		const int j0 = static_cast<int>(r - static_cast<long long>(i) * quads) * 4;
		float *x = reinterpret_cast<float *>(static_cast<char *>(L.planes[p]) + static_cast<ptrdiff_t>(i) * L.stride);
		const float *a = reinterpret_cast<const float *>(static_cast<const char *>(L.alpha) +
		                                                 static_cast<ptrdiff_t>(i) * L.alpha_stride);
		const int n = min(4, L.width - j0);
		for (int e = 0; e < n; ++e) {
			const float v = x[j0 + e], al = a[j0 + e];
			if (INVERSE) {
				// alpha clamped to [0, 1] (a NaN passes), 0 where it is 0
				const float c = al < 0.0f ? 0.0f : (1.0f < al ? 1.0f : al);
				x[j0 + e] = c == 0.0f ? 0.0f : __fdiv_rn(v, c);
			} else {
				// zimg multiplies by the alpha sample as it is (its clamped
				// copy goes unused, simple_filters.cpp:83-85)
				x[j0 + e] = __fmul_rn(v, al);
			}
		}
	}
}

__global__ void __launch_bounds__(kThreads) fill_kernel(void *dst, ptrdiff_t stride, int width, int height, int bytes,
                                                      uint32_t value)
{
	const long long total = static_cast<long long>(width) * height;
	for (long long u = static_cast<long long>(blockIdx.x) * kThreads + threadIdx.x; u < total;
	     u += static_cast<long long>(gridDim.x) * kThreads) {
		const int i = static_cast<int>(u / width), j = static_cast<int>(u - static_cast<long long>(i) * width);
		char *row = static_cast<char *>(dst) + static_cast<ptrdiff_t>(i) * stride;
		if (bytes == 1)
			reinterpret_cast<uint8_t *>(row)[j] = static_cast<uint8_t>(value);
		else if (bytes == 2)
			reinterpret_cast<uint16_t *>(row)[j] = static_cast<uint16_t>(value);
		else
			reinterpret_cast<uint32_t *>(row)[j] = value;
	}
}

int grid_for(long long units)
{
	static int sms = 0;
	if (!sms) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (sms < 1)
			sms = 1;
	}
	return static_cast<int>(std::min<long long>((units + kThreads - 1) / kThreads, static_cast<long long>(sms) * 8));
}

} // namespace

cudaError_t launch_fill(void *dst, ptrdiff_t stride, int width, int height, int bytes, uint32_t value,
                        cudaStream_t stream)
{
	if (width <= 0 || height <= 0)
		return cudaSuccess;
	if (bytes != 1 && bytes != 2 && bytes != 4)
		return cudaErrorInvalidValue;
	fill_kernel<<<grid_for(static_cast<long long>(width) * height), kThreads, 0, stream>>>(dst, stride, width, height,
	                                                                                      bytes, value);
	return cudaGetLastError();
}

cudaError_t launch_alpha(const AlphaLaunch &L, bool inverse, cudaStream_t stream)
{
	if (L.width <= 0 || L.height <= 0 || L.num_planes <= 0)
		return cudaSuccess;
	if (L.num_planes > 3)
		return cudaErrorInvalidValue;
	const int grid = grid_for(static_cast<long long>((L.width + 3) / 4) * L.height * L.num_planes);
	if (inverse)
		alpha_kernel<true><<<grid, kThreads, 0, stream>>>(L);
	else
		alpha_kernel<false><<<grid, kThreads, 0, stream>>>(L);
	return cudaGetLastError();
}

} // namespace zg
