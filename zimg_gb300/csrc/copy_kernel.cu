// Batched plane copies: every identity conversion of a batch in one launch.
#include <algorithm>

#include "kernels.h"

namespace zg {

namespace {

__global__ void __launch_bounds__(256)
plane_copy_kernel(const PlaneCopy *__restrict__ t, int n, unsigned long long total)
{
	for (unsigned long long c = blockIdx.x * 256ull + threadIdx.x; c < total; c += gridDim.x * 256ull) {
		int lo = 0, hi = n - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (t[mid].chunk_begin <= c)
				lo = mid;
			else
				hi = mid - 1;
		}
		const PlaneCopy &p = t[lo];
		const unsigned long long local = c - p.chunk_begin;
		const unsigned row = static_cast<unsigned>(local / p.chunks_per_row);
		const unsigned off = static_cast<unsigned>(local - static_cast<unsigned long long>(row) * p.chunks_per_row) * p.unit;
		const char *s = static_cast<const char *>(p.src) + static_cast<ptrdiff_t>(row) * p.src_stride + off;
		char *d = static_cast<char *>(p.dst) + static_cast<ptrdiff_t>(row) * p.dst_stride + off;
		if (p.unit == 16)
			*reinterpret_cast<uint4 *>(d) = __ldg(reinterpret_cast<const uint4 *>(s));
		else if (p.unit == 4)
			*reinterpret_cast<uint32_t *>(d) = __ldg(reinterpret_cast<const uint32_t *>(s));
		else
			*reinterpret_cast<uint16_t *>(d) = __ldg(reinterpret_cast<const uint16_t *>(s));
	}
}

} // namespace

cudaError_t launch_plane_copies(const PlaneCopy *table, int n, unsigned long long total_chunks, cudaStream_t stream)
{
	if (!n || !total_chunks)
		return cudaSuccess;
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const unsigned long long want = (total_chunks + 255) / 256;
	const unsigned grid = static_cast<unsigned>(std::min<unsigned long long>(want, static_cast<unsigned long long>(std::max(1, sms)) * 8));
	plane_copy_kernel<<<grid, 256, 0, stream>>>(table, n, total_chunks);
	return cudaGetLastError();
}

} // namespace zg
