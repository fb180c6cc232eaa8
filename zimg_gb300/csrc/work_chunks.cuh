// Guided work chunks of a persistent launch (WorkChunks, fused.h): the CTAs
// of a launch take chunks of its work units from one counter, in the order
// they ask, until none is left; the last CTA out leaves the counter zero for
// the next launch on the same stream (or the next replay of a graph).
#pragma once

#include "fused.h"

namespace zg {

// The next chunk for this CTA (the same value in every thread), or -1 when
// every chunk is taken. `slot`: a shared-memory int of the CTA. Every thread
// of the CTA calls it.
__device__ __forceinline__ int next_chunk(const WorkChunks &C, int *slot)
{
	if (threadIdx.x == 0)
		*slot = static_cast<int>(atomicAdd(&C.sched[0], 1u));
	__syncthreads();
	const int m = *slot;
	__syncthreads();  // every thread has read it before thread 0 asks again
	return m < C.num ? m : -1;
}

// Called by every CTA once, after its last chunk (thread 0 acts).
__device__ __forceinline__ void chunks_finish(const WorkChunks &C)
{
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(&C.sched[1], 1u) == gridDim.x - 1) {
			atomicExch(&C.sched[0], 0u);
			atomicExch(&C.sched[1], 0u);
		}
	}
}

} // namespace zg
