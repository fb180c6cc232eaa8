// Issue model of tcgen05.mma.kind::tf32 (M = 128, K = 8, cta_group::1):
// cycles per instruction for several N, numbers of rotating accumulators, and
// A from tensor memory (ts) or shared memory (ss). One CTA, one issuing
// thread, operands zero; the completion wait is bounded (about 1 s of clock).
// Output: one line per configuration, "N acc ts|ss issue complete MAC/clk".
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t desc(unsigned a, unsigned lbo, unsigned sbo) {
  return (uint64_t)((a >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
__device__ __forceinline__ uint32_t idesc(int n) { return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24); }

__global__ void probe(int n, int nacc, int ts, int iters, unsigned long long *out, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  int tid = threadIdx.x;
  // zero A (4 KB) and B (n x 8 x 4 bytes) in shared memory
  for (int i = tid; i < (4096 + 8192) / 4; i += blockDim.x) ((uint32_t *)sm)[i] = 0;
  if (tid == 0) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bar))); asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" :: "r"(saddr(&slot)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t tm = slot;
  if (tid == 0) {
    const unsigned a_s = saddr(sm), b_s = saddr(sm + 4096);
    const uint64_t da = desc(a_s, 128 * 16, 128), db = desc(b_s, 128 * (n / 8), 128);
    const uint32_t id = idesc(n);
    long long t0 = clock64();
    for (int i = 0; i < iters; ++i) {
      uint32_t d = tm + 256 + (uint32_t)((i % nacc) * n);
      uint32_t acc = i >= nacc;
      if (ts)
        asm volatile("{.reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;}" :: "r"(d), "r"(tm), "l"(db), "r"(id), "r"(acc) : "memory");
      else
        asm volatile("{.reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;}" :: "r"(d), "l"(da), "l"(db), "r"(id), "r"(acc) : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(saddr(&bar)) : "memory");
    long long t1 = clock64();
    unsigned done = 0;
    for (long long k = 0; !done && clock64() - t1 < 2000000000LL; ++k) {
      asm volatile("{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p;}" : "=r"(done) : "r"(saddr(&bar)) : "memory");
    }
    long long t2 = clock64();
    if (!done) *err = 1;
    out[0] = t1 - t0; out[1] = t2 - t0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid < 32) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" :: "r"(tm) : "memory");
  }
}

int main() {
  unsigned long long *out; int *err;
  cudaMalloc(&out, 16); cudaMalloc(&err, 4); cudaMemset(err, 0, 4);
  cudaFuncSetAttribute(probe, cudaFuncAttributeMaxDynamicSharedMemorySize, 16384);
  struct { int n, nacc, ts; } cfg[] = {{16,1,1},{16,8,1},{16,1,0},{16,8,0},{32,1,1},{32,8,1},{64,1,1},{64,4,1},{128,1,1},{128,2,1},{256,1,1},{256,1,0}};
  const int iters = 4096;
  for (auto c : cfg) {
    probe<<<1, 128, 16384>>>(c.n, c.nacc, c.ts, iters, out, err);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[2]; int he = 0;
    cudaMemcpy(h, out, 16, cudaMemcpyDeviceToHost); cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost);
    printf("N=%3d acc=%d %s: issue %.1f cyc/mma, complete %.1f cyc/mma, %.0f MAC/clk  err=%d %s\n", c.n, c.nacc, c.ts ? "ts" : "ss",
           (double)h[0] / iters, (double)h[1] / iters, 128.0 * c.n * 8 * iters / h[1], he, cudaGetErrorString(e));
    if (e != cudaSuccess || he) return 1;
  }
  return 0;
}
