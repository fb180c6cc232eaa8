// mbarrier and bulk-copy helpers shared by the TMA-pipelined kernels
// (PTX ISA: mbarrier, cp.async.bulk, cp.async.bulk.tensor).
#pragma once

#include <cstdint>

namespace zg {

constexpr unsigned long long kWaitNs = 250000000ull;  // a pipeline wait gives up after 0.25 s

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
	return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
	             : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
	return t;
}

// Wait until the phase of the given parity has completed; false when the
// wait has lasted kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
	const unsigned a = smem_addr(bar);
	unsigned long long t0 = 0;
	for (unsigned i = 0;; ++i) {
		unsigned done;
		asm volatile("{\n"
		             "  .reg .pred p;\n"
		             "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
		             "  selp.u32 %0, 1, 0, p;\n"
		             "}\n"
		             : "=r"(done)
		             : "r"(a), "r"(parity)
		             : "memory");
		if (done)
			return true;
		if ((i & 63) == 0) {
			const unsigned long long t = global_ns();
			if (i == 0)
				t0 = t;
			else if (t - t0 > kWaitNs)
				return false;
		}
	}
}

// One box of the tensor map at (x, y) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, int x, int y, uint64_t *bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
	                 smem_addr(dst)),
	             "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar))
	             : "memory");
}

// `bytes` contiguous bytes (16-byte aligned, a multiple of 16) into shared memory.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
	                 smem_addr(dst)),
	             "l"(src), "r"(bytes), "r"(smem_addr(bar))
	             : "memory");
}

} // namespace zg
