// FP32 wide-filter passes (strong downscales, tens to hundreds of taps per
// output) on the fifth-generation tensor cores: the banded product of
// wide_kernel.cu with the split samples in tensor memory, the taps in shared
// memory and the accumulators in tensor memory (tcgen05.mma with A from
// TMEM), fed by tensor copies.
//
// A pass computes out[o][m] = sum_k tap(o, k) * in[k][m] for every output o
// along the filtered axis and every line m across it (m = column of a
// vertical pass, row of a horizontal one). A work item is a tile of 128
// lines times a group of 16 outputs; the group's band of inputs is cut into
// chunks of 32. Per chunk:
//
//  - a producer lane copies the 32 x 128 tile of input samples
//    (cp.async.bulk.tensor; zeros outside the plane) and the chunk's tap
//    block (cp.async.bulk) into a stage of a ring;
//  - 8 converter warps, two per TMEM lane quadrant, read their lines'
//    samples, split each into a TF32 high part and a TF32 remainder
//    (3xTF32) and store both into tensor memory (tcgen05.st; TMEM lane =
//    line, column = input): the A operands of the chunk;
//  - one MMA lane issues, per 8 inputs, the products lo*hi, hi*lo and hi*hi
//    (tcgen05.mma.cta_group::1.kind::tf32, A from tensor memory, B from
//    shared memory, M = 128 lines, N = 16 outputs, K = 8) into one of 8
//    tensor-memory accumulators, from zero per chunk;
//  - 4 epilogue warps read the chunk's accumulator (tcgen05.ld) and add it to
//    their running sums in fp32, and store their line's 16 outputs when the
//    band ends.
//
// Shared memory carries each sample twice (the tensor copy's write, the
// converter's read); the operands the tensor core re-reads for its three
// products come from tensor memory.
//
// Split: hi = x with its 13 low mantissa bits cleared (truncation to TF32),
// lo = x - hi (exact) rounded to nearest TF32 by integer arithmetic on its
// bits; each product keeps about 21 significant bits. A non-finite sample
// gives lo = NaN, so its outputs are NaN. Chunk sums are added with ordinary
// fp32 adds, in chunk order: the tensor core's internal additions are not
// round-to-nearest, and one accumulator carried through a whole 600-tap band
// measured 7x the C path's error (resize_impl.cpp:61-114) against FP64,
// where chunks of 32 inputs stay below it.
//
// Input tiles: a vertical pass copies 32 rows x 128 columns (raw[input][line],
// 512-byte rows), a horizontal pass 128 rows x 32 columns with the 128-byte
// swizzle (16-byte chunk c of line r at chunk c ^ (r % 8)), so that the 8
// lines a quarter-warp reads fall in different shared-memory banks.
//
// Tap blocks (B, 16 outputs x 32 inputs, built on the host) use the K-major
// no-swizzle layout of the tcgen05 shared memory descriptors: core matrices
// of 8 outputs x 4 inputs (128 contiguous bytes), (output / 8) * 128 +
// (input / 4) * 256; the descriptor's leading byte offset is the stride
// between core matrices along K (256), its stride byte offset the stride
// between groups of 8 outputs (128).
//
// Every mbarrier wait is bounded (kWaitNs). A wait that runs out records its
// cause in g_wide_pipeline_error, the CTA stops, the producer waits (bounded)
// for the copies it has in flight, and tensor memory is freed.
#include <cuda.h>

#include <algorithm>

#include "fused.h"
#include "kernels.h"
#include "pipeline.cuh"

namespace zg {

namespace {

constexpr int kM = 128;                 // lines per tile: TMEM lanes
constexpr int kN = 16;                  // outputs per group
constexpr int kKC = 32;                 // inputs per chunk
constexpr int kStages = 8;              // ring of input tiles
constexpr int kRegions = 8;             // TMEM accumulators of kN columns
constexpr int kConvWarps = 8;
constexpr int kEpiWarps = 4;
constexpr int kThreads = (2 + kEpiWarps + kConvWarps) * 32;  // producer, MMA, epilogue, converters

// tensor memory columns: A operands of two chunks (hi 32 | lo 32 each), then
// the accumulators
constexpr uint32_t kColA = 0;
constexpr uint32_t kColD = 2 * 2 * kKC;
constexpr uint32_t kTmemCols = 256;
static_assert(kColD + kRegions * kN <= kTmemCols, "tensor memory columns");

constexpr unsigned kLboB = 256;
constexpr unsigned kSboB = 128;
constexpr unsigned kRawBytes = kKC * kM * 4;      // input tile
constexpr unsigned kBBytes = 2 * kN * kKC * 4;    // tap block: hi | lo
constexpr unsigned kStageBytes = kRawBytes + kBBytes;
constexpr unsigned kOffBar = kStages * kStageBytes;
constexpr unsigned kNumBars = 3 * kStages + 4 + 2 * kRegions + 1;
constexpr unsigned kSmemBytes = kOffBar + kNumBars * 8 + 16 + 1024;  // + TMEM address slot, base alignment

// kind::tf32 instruction descriptor: D f32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(kN >> 3) << 17) |
                            (static_cast<uint32_t>(kM >> 4) << 24);

static_assert(kStageBytes % 1024 == 0, "swizzled tensor copies land on 1024-byte boundaries");
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");

__device__ int g_wide_pipeline_error;

struct UmmaPass {
	const uint4 *chunk;        // tap blocks, kBBytes each
	const int *chunk_begin;    // per group; [groups] = number of chunks
	const int *kbase;          // per group
	int groups;
	int items;                 // line tiles x groups
	int m_extent;              // lines
	int dst_dim;               // outputs
	char *dst;
	ptrdiff_t dm;              // bytes between lines of the destination
	ptrdiff_t dko;             // bytes between outputs of the destination
};

// Shared memory descriptor (no swizzle, version 1 at bits 46-47).
__device__ __forceinline__ uint64_t umma_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
	return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
	       (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D (TMEM) (+)= A (TMEM) * B (shared memory).
__device__ __forceinline__ void umma_tf32_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t accumulate)
{
	asm volatile("{\n"
	             "  .reg .pred p;\n"
	             "  setp.ne.b32 p, %4, 0;\n"
	             "  tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n"
	             "}\n" ::"r"(d),
	             "r"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
	             : "memory");
}

// Arrive on bar once every tcgen05 operation this thread issued has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
	             : "memory");
}

__device__ __forceinline__ void tc_fence_before()
{
	asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
	asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// 16 consecutive columns of this warp's 32 TMEM lanes, one lane per thread;
// the load and its wait in one statement so that no use of the values is
// scheduled before the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
	             "%14, %15}, [%16];\n"
	             "tcgen05.wait::ld.sync.aligned;\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
	               "=r"(r[15])
	             : "r"(taddr)
	             : "memory");
#pragma unroll
	for (int i = 0; i < 16; ++i)
		v[i] = __uint_as_float(r[i]);
}

// 16 consecutive columns of this warp's 32 TMEM lanes from registers.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16])
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
	             "%13, %14, %15, %16};\n" ::"r"(taddr),
	             "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
	             "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
	             : "memory");
}

__device__ __forceinline__ void tmem_st_wait()
{
	asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
}

// x -> (TF32 high part by truncation, remainder rounded to nearest TF32).
__device__ __forceinline__ void split(float x, uint32_t &hi, uint32_t &lo)
{
	hi = __float_as_uint(x) & 0xFFFFE000u;
	lo = (__float_as_uint(x - __uint_as_float(hi)) + 0x1000u) & 0xFFFFE000u;
}

__device__ __forceinline__ void record_failure(int cause, volatile int *abort_flag)
{
	atomicCAS(&g_wide_pipeline_error, 0, cause);
	*abort_flag = 1;
}

// HORIZ: horizontal pass (tile = 128 rows x 32 columns of the source,
// swizzled); otherwise vertical (32 rows x 128 columns).
template <bool HORIZ>
__global__ void __launch_bounds__(kThreads, 1)
wide_umma_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ UmmaPass p)
{
	extern __shared__ unsigned char smem_dyn[];
	__shared__ int abort_word;
	volatile int *abort_flag = &abort_word;
	unsigned char *sm =
		reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~static_cast<uintptr_t>(1023));
	uint64_t *raw_full = reinterpret_cast<uint64_t *>(sm + kOffBar);
	uint64_t *raw_empty = raw_full + kStages;   // the converters are done with the samples
	uint64_t *b_empty = raw_empty + kStages;    // the MMAs are done with the taps
	uint64_t *a_full = b_empty + kStages;
	uint64_t *a_empty = a_full + 2;
	uint64_t *t_full = a_empty + 2;
	uint64_t *t_empty = t_full + kRegions;
	uint64_t *done = t_empty + kRegions;
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

	if (threadIdx.x == 0) {
		for (int s = 0; s < kStages; ++s) {
			mbar_init(&raw_full[s], 1);
			mbar_init(&raw_empty[s], kConvWarps);
			mbar_init(&b_empty[s], 1);
		}
		for (int b = 0; b < 2; ++b) {
			mbar_init(&a_full[b], kConvWarps);
			mbar_init(&a_empty[b], 1);
		}
		for (int r = 0; r < kRegions; ++r) {
			mbar_init(&t_full[r], 1);
			mbar_init(&t_empty[r], kEpiWarps);
		}
		mbar_init(done, 1);
		*abort_flag = 0;
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tmem_slot)),
		             "r"(kTmemCols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	const long long i0 = static_cast<long long>(blockIdx.x) * p.items / gridDim.x;
	const long long i1 = static_cast<long long>(blockIdx.x + 1) * p.items / gridDim.x;

	if (warp == 0) {
		if (lane == 0) {
			// producer
			asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmap) : "memory");
			unsigned seq = 0;
			bool ok = true;
			for (long long it = i0; ok && it < i1; ++it) {
				const int g = static_cast<int>(it % p.groups), mt = static_cast<int>(it / p.groups);
				const int c0 = __ldg(p.chunk_begin + g), nc = __ldg(p.chunk_begin + g + 1) - c0;
				const int kb = __ldg(p.kbase + g);
				for (int c = 0; c < nc; ++c, ++seq) {
					const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
					if (*abort_flag || !mbar_wait(&raw_empty[st], ph ^ 1) || !mbar_wait(&b_empty[st], ph ^ 1)) {
						if (!*abort_flag)
							record_failure(2, abort_flag);
						ok = false;
						break;
					}
					unsigned char *stage = sm + st * kStageBytes;
					mbar_arrive_expect_tx(&raw_full[st], kStageBytes);
					if (HORIZ)
						tma_load_2d(stage, &tmap, kb + kKC * c, mt * kM, &raw_full[st]);
					else
						tma_load_2d(stage, &tmap, mt * kM, kb + kKC * c, &raw_full[st]);
					bulk_load(stage + kRawBytes, p.chunk + static_cast<size_t>(c0 + c) * (kBBytes / 16), kBBytes,
					          &raw_full[st]);
				}
			}
			if (!ok) {
				// the copies still in flight: the last one issued into each stage
				for (unsigned j = seq > kStages ? seq - kStages : 0; j < seq; ++j)
					mbar_wait(&raw_full[j % kStages], (j / kStages) & 1);
			}
		}
	} else if (warp == 1) {
		if (lane == 0) {
			// MMA issue
			const unsigned sbase = smem_addr(sm);
			unsigned seq = 0;
			bool ok = true;
			for (long long it = i0; ok && it < i1; ++it) {
				const int g = static_cast<int>(it % p.groups);
				const int nc = __ldg(p.chunk_begin + g + 1) - __ldg(p.chunk_begin + g);
				for (int c = 0; c < nc; ++c, ++seq) {
					const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
					const unsigned ab = seq & 1, aph = (seq >> 1) & 1;
					const unsigned r = seq % kRegions, rph = (seq / kRegions) & 1;
					if (*abort_flag || !mbar_wait(&a_full[ab], aph) || !mbar_wait(&raw_full[st], ph) ||
					    !mbar_wait(&t_empty[r], rph ^ 1)) {
						if (!*abort_flag)
							record_failure(3, abort_flag);
						ok = false;
						break;
					}
					tc_fence_after();
					const uint32_t d = tmem + kColD + r * kN;
					const uint32_t ahi = tmem + kColA + ab * 2 * kKC, alo = ahi + kKC;
					const unsigned bhi = sbase + st * kStageBytes + kRawBytes, blo = bhi + kBBytes / 2;
#pragma unroll
					for (int s = 0; s < kKC / 8; ++s) {
						const uint64_t db_hi = umma_desc(bhi + 2 * s * kLboB, kLboB, kSboB);
						const uint64_t db_lo = umma_desc(blo + 2 * s * kLboB, kLboB, kSboB);
						umma_tf32_ts(d, alo + 8 * s, db_hi, s > 0);
						umma_tf32_ts(d, ahi + 8 * s, db_lo, 1);
						umma_tf32_ts(d, ahi + 8 * s, db_hi, 1);
					}
					umma_commit(&a_empty[ab]);
					umma_commit(&b_empty[st]);
					umma_commit(&t_full[r]);
				}
			}
			// nothing of this CTA's may still read shared or tensor memory on return
			umma_commit(done);
			if (!mbar_wait(done, 0))
				record_failure(3, abort_flag);
		}
	} else if (warp < 2 + kEpiWarps) {
		// epilogue: TMEM lanes 32 q .. 32 q + 31 belong to warp q of a warpgroup
		const int q = warp & 3;
		const uint32_t tl = tmem + (static_cast<uint32_t>(32 * q) << 16);
		const int ml = 32 * q + lane;
		unsigned seq = 0;
		bool ok = true;
		for (long long it = i0; ok && it < i1; ++it) {
			const int g = static_cast<int>(it % p.groups), mt = static_cast<int>(it / p.groups);
			const int nc = __ldg(p.chunk_begin + g + 1) - __ldg(p.chunk_begin + g);
			float sum[kN];
#pragma unroll
			for (int n = 0; n < kN; ++n)
				sum[n] = 0.0f;
			for (int c = 0; c < nc; ++c, ++seq) {
				const unsigned r = seq % kRegions, rph = (seq / kRegions) & 1;
				if (__any_sync(0xffffffffu, *abort_flag) || !__all_sync(0xffffffffu, mbar_wait(&t_full[r], rph))) {
					if (lane == 0 && !*abort_flag)
						record_failure(4, abort_flag);
					ok = false;
					break;
				}
				tc_fence_after();
				float v[kN];
				tmem_ld16(tl + kColD + r * kN, v);
				tc_fence_before();
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&t_empty[r]);
#pragma unroll
				for (int n = 0; n < kN; ++n)
					sum[n] += v[n];
			}
			if (!ok)
				break;
			const int m = mt * kM + ml;
			if (m < p.m_extent) {
				const int o0 = g * kN;
				char *d = p.dst + static_cast<ptrdiff_t>(m) * p.dm + static_cast<ptrdiff_t>(o0) * p.dko;
#pragma unroll
				for (int n = 0; n < kN; ++n)
					if (o0 + n < p.dst_dim)
						*reinterpret_cast<float *>(d + n * p.dko) = sum[n];
			}
		}
	} else {
		// converters: warp (quadrant q, half h) splits inputs 16 h .. 16 h + 15
		// of lines 32 q .. 32 q + 31
		const int cw = warp - 2 - kEpiWarps;
		const int q = warp & 3, h = cw >> 2;
		const int m = 32 * q + lane;
		const uint32_t tl = tmem + (static_cast<uint32_t>(32 * q) << 16) + kColA + 16 * h;
		unsigned seq = 0;
		bool ok = true;
		for (long long it = i0; ok && it < i1; ++it) {
			const int g = static_cast<int>(it % p.groups);
			const int nc = __ldg(p.chunk_begin + g + 1) - __ldg(p.chunk_begin + g);
			for (int c = 0; c < nc; ++c, ++seq) {
				const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
				const unsigned ab = seq & 1, aph = (seq >> 1) & 1;
				if (__any_sync(0xffffffffu, *abort_flag) ||
				    !__all_sync(0xffffffffu, mbar_wait(&raw_full[st], ph) && mbar_wait(&a_empty[ab], aph ^ 1))) {
					if (lane == 0 && !*abort_flag)
						record_failure(1, abort_flag);
					ok = false;
					break;
				}
				const unsigned char *raw = sm + st * kStageBytes;
				float x[16];
				if (HORIZ) {
					// line m: 128 bytes, 16-byte chunk j at chunk j ^ (m % 8)
#pragma unroll
					for (int i = 0; i < 4; ++i) {
						const float4 v = *reinterpret_cast<const float4 *>(raw + m * 128 + (((4 * h + i) ^ (m & 7)) << 4));
						x[4 * i] = v.x;
						x[4 * i + 1] = v.y;
						x[4 * i + 2] = v.z;
						x[4 * i + 3] = v.w;
					}
				} else {
#pragma unroll
					for (int j = 0; j < 16; ++j)
						x[j] = reinterpret_cast<const float *>(raw)[(16 * h + j) * kM + m];
				}
				uint32_t hi[16], lo[16];
#pragma unroll
				for (int j = 0; j < 16; ++j)
					split(x[j], hi[j], lo[j]);
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&raw_empty[st]);
				tc_fence_after();
				tmem_st16(tl + ab * 2 * kKC, hi);
				tmem_st16(tl + ab * 2 * kKC + kKC, lo);
				tmem_st_wait();
				tc_fence_before();
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&a_full[ab]);
			}
		}
	}

	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		__syncwarp();
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
	}
}

int sm_count_umma()
{
	int dev = 0, n = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
	return n > 0 ? n : 152;
}

template <bool HORIZ>
cudaError_t set_smem_attr()
{
	return cudaFuncSetAttribute(wide_umma_kernel<HORIZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                            static_cast<int>(kSmemBytes));
}

} // namespace

cudaError_t launch_wide_umma(const PassLaunch &l, cudaStream_t stream)
{
	const WideTables &w = l.wide;
	if (!w.uchunk || l.src_stride <= 0 || reinterpret_cast<uintptr_t>(l.src) % 16 || l.src_stride % 16)
		return cudaErrorNotSupported;
	const uint64_t src_dim = l.t.input_width, lines = l.lines;
	CUtensorMap map;
	const bool ok = l.horizontal
	                    ? encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, l.src, src_dim, lines,
	                                           static_cast<uint64_t>(l.src_stride), kKC, kM, true)
	                    : encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, l.src, lines, src_dim,
	                                           static_cast<uint64_t>(l.src_stride), kM, kKC, false);
	if (!ok)
		return cudaErrorNotSupported;
	UmmaPass p{};
	p.chunk = w.uchunk;
	p.chunk_begin = w.uchunk_begin;
	p.kbase = w.ukbase;
	p.groups = w.ugroups;
	p.items = static_cast<int>((lines + kM - 1) / kM) * w.ugroups;
	p.m_extent = static_cast<int>(lines);
	p.dst_dim = static_cast<int>(l.t.rows);
	p.dst = static_cast<char *>(l.dst);
	p.dm = l.horizontal ? l.dst_stride : 4;
	p.dko = l.horizontal ? 4 : l.dst_stride;
	if (p.items <= 0)
		return cudaSuccess;
	const int grid = std::min(p.items, sm_count_umma());
	cudaError_t e = l.horizontal ? set_smem_attr<true>() : set_smem_attr<false>();
	if (e != cudaSuccess)
		return e;
	if (l.horizontal)
		wide_umma_kernel<true><<<grid, kThreads, kSmemBytes, stream>>>(map, p);
	else
		wide_umma_kernel<false><<<grid, kThreads, kSmemBytes, stream>>>(map, p);
	return cudaGetLastError();
}

int wide_umma_pipeline_error(bool reset)
{
	int v = 0;
	if (cudaMemcpyFromSymbol(&v, g_wide_pipeline_error, sizeof(v)) != cudaSuccess)
		return -1;
	if (reset && v) {
		const int zero = 0;
		cudaMemcpyToSymbol(g_wide_pipeline_error, &zero, sizeof(zero));
	}
	return v;
}

} // namespace zg
