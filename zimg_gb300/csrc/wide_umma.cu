// FP32 vertical wide-filter passes (strong downscales, tens to about 160 taps
// per output) on the fifth-generation tensor cores (tcgen05.mma, operands in
// shared memory, accumulators in tensor memory), fed by tensor copies.
//
// A pass computes out[o][x] = sum_k tap(o, k) * in[k][x] for every output row
// o and column x. The product is laid out for the tensor core's issue model:
// a tcgen05.mma.kind::tf32 of M = 128, K = 8 costs about 200 cycles whatever
// its N (measured, 16 <= N <= 256), so N carries 256 image columns and M the
// taps of 64 outputs twice, their TF32 high parts in rows 0-63 and their TF32
// remainders in rows 64-127. A work item is one tile of 256 columns x 64
// outputs; its band of input rows is cut into chunks of 16 rows. Per chunk:
//
//  - a producer lane copies the 16 x 256 tile of samples
//    (cp.async.bulk.tensor; zeros outside the plane) and the chunk's tap
//    blocks (cp.async.bulk, built on the host) into a stage of a ring;
//  - 8 converter warps split each sample into a TF32 high part (truncation)
//    and a TF32 remainder (rounded to nearest by integer arithmetic on its
//    bits) and write both into the K-major operand layout (core matrices of
//    8 rows x 4 inputs); the MMAs read the tap blocks in the stage, which is
//    refilled once both the converters and those MMAs are done with it;
//  - one MMA lane issues per 8 input rows D += A * X_hi and D += A * X_lo
//    (M = 128, N = 256, K = 8), accumulating the whole band of the tile in
//    one of two tensor-memory accumulators: row i < 64 of D is the sum of
//    tap_hi * x over the band, row 64 + i the sum of tap_lo * x;
//  - 4 epilogue warps read the accumulator (tcgen05.ld, TMEM lane = row),
//    add row 64 + i to row i in fp32 through shared memory, and store output
//    o0 + i of the tile's 256 columns.
//
// Each output row sees nonzero taps only within its own band (at most
// kUmmaMaxTaps inputs: 2 * ceil(taps / 8) + 2 accumulating products); rows
// outside it add exact zeros. A non-finite sample gives a NaN remainder, so
// its outputs are NaN.
//
// Operand layouts (PTX ISA, tcgen05 shared memory descriptors, K-major, no
// swizzle): a core matrix is 8 rows x 16 bytes (4 TF32 values along K), 128
// contiguous bytes; the descriptor's leading byte offset is the stride
// between core matrices along K, its stride byte offset the stride between
// groups of 8 rows (128 bytes in both operands). Taps (A, 128 rows x 8
// inputs per 8-row block): core matrix (row / 8, input / 4) at (row / 8) *
// 128 + (input / 4) * 2048. Samples (B, 256 columns x 16 inputs per chunk):
// core matrix (column / 8, input / 4) at (column / 8) * 128 + (input / 4) *
// kLboX, kLboX = 32 core matrices plus 16 bytes, so that the 4 core matrices
// a converter lane writes fall in different banks.
//
// Every mbarrier wait is bounded (kWaitNs). A wait that runs out records its
// cause in g_wide_pipeline_error, the CTA stops, the producer waits (bounded)
// for the copies it has in flight, the MMA lane for its products, and tensor
// memory is freed.
#include <cuda.h>

#include <algorithm>

#include "fused.h"
#include "kernels.h"
#include "pipeline.cuh"

namespace zg {

namespace {

constexpr int kCols = 256;              // image columns per tile: N
constexpr int kOut = 64;                // outputs per tile; M = 2 * kOut
constexpr int kKC = 16;                 // input rows per chunk
constexpr int kStages = 6;              // ring of sample tiles
constexpr int kConvWarps = 8;
constexpr int kEpiWarps = 4;
constexpr int kThreads = (2 + kEpiWarps + kConvWarps) * 32;  // producer, MMA, epilogue, converters
constexpr uint32_t kTmemCols = 512;     // two accumulators of kCols columns

constexpr unsigned kSbo = 128;
constexpr unsigned kLboA = 2048;
constexpr unsigned kLboX = (kCols / 8) * 128 + 16;
constexpr unsigned kRawBytes = kKC * kCols * 4;            // sample tile, raw[row][column]
constexpr unsigned kABytes = (kKC / 8) * 2 * kOut * 8 * 4; // tap blocks of a chunk
constexpr unsigned kStageBytes = kRawBytes + kABytes;
constexpr unsigned kXOp = (kKC / 4) * kLboX;               // one sample operand (hi or lo)
constexpr unsigned kXBuf = 2 * kXOp;                       // hi | lo
constexpr unsigned kXchStride = 36;                        // floats per exchanged row
constexpr unsigned kXchBytes = 2 * 32 * kXchStride * 4;
constexpr unsigned kOffX = kStages * kStageBytes;
constexpr unsigned kOffXch = kOffX + 2 * kXBuf;
constexpr unsigned kOffBar = kOffXch + kXchBytes;
constexpr unsigned kNumBars = 2 * kStages + 4 + 4 + 1;
constexpr unsigned kSmemBytes = kOffBar + kNumBars * 8 + 16 + 1024;  // + TMEM address slot, base alignment

// kind::tf32 instruction descriptor: D f32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(kCols >> 3) << 17) |
                            (static_cast<uint32_t>((2 * kOut) >> 4) << 24);

static_assert(kStageBytes % 128 == 0 && kXBuf % 16 == 0 && kXOp % 16 == 0, "copy and operand alignment");
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");

__device__ int g_wide_pipeline_error;

struct UmmaPass {
	const uint4 *chunk;        // tap blocks, kABytes per chunk
	const int *chunk_begin;    // per tile; [tiles] = number of chunks
	const int *kbase;          // per tile
	int tiles;                 // output tiles
	int items;                 // column tiles x output tiles
	int columns;               // plane width
	int dst_dim;               // output rows
	char *dst;
	ptrdiff_t dst_stride;
	int dst_aligned;           // dst and dst_stride multiples of 16 bytes
};

// Shared memory descriptor (no swizzle, version 1 at bits 46-47).
__device__ __forceinline__ uint64_t umma_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
	return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
	       (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void umma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate)
{
	asm volatile("{\n"
	             "  .reg .pred p;\n"
	             "  setp.ne.b32 p, %4, 0;\n"
	             "  tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
	             "}\n" ::"r"(d),
	             "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
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

// 32 consecutive columns of this warp's 32 TMEM lanes, one lane per thread;
// the load and its wait in one statement so that no use of the values is
// scheduled before the wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
	uint32_t r[32];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
	             "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
	             "tcgen05.wait::ld.sync.aligned;\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
	               "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
	               "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
	               "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	             : "r"(taddr)
	             : "memory");
#pragma unroll
	for (int i = 0; i < 32; ++i)
		v[i] = __uint_as_float(r[i]);
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

__device__ __forceinline__ void epilogue_sync()
{
	asm volatile("bar.sync 1, %0;\n" ::"n"(kEpiWarps * 32) : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
wide_umma_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ UmmaPass p)
{
	extern __shared__ unsigned char smem_dyn[];
	__shared__ int abort_word, epi_fail_word;
	volatile int *abort_flag = &abort_word;
	volatile int *epi_fail = &epi_fail_word;  // set before an epilogue barrier, read after it
	// 1024-byte aligned base, as an offset from the shared array so that every
	// access through it stays a shared-memory access
	unsigned char *sm = smem_dyn + ((1024u - (smem_addr(smem_dyn) & 1023u)) & 1023u);
	uint64_t *raw_full = reinterpret_cast<uint64_t *>(sm + kOffBar);
	uint64_t *raw_empty = raw_full + kStages;
	uint64_t *x_full = raw_empty + kStages;
	uint64_t *x_empty = x_full + 2;
	uint64_t *d_full = x_empty + 2;
	uint64_t *d_empty = d_full + 2;
	uint64_t *done = d_empty + 2;
	uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
	float *xch = reinterpret_cast<float *>(sm + kOffXch);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

	if (threadIdx.x == 0) {
		for (int s = 0; s < kStages; ++s) {
			mbar_init(&raw_full[s], 1);
			mbar_init(&raw_empty[s], kConvWarps + 1);  // the converters, then the MMAs that read the tap blocks
		}
		for (int b = 0; b < 2; ++b) {
			mbar_init(&x_full[b], kConvWarps);
			mbar_init(&x_empty[b], 1);
			mbar_init(&d_full[b], 1);
			mbar_init(&d_empty[b], kEpiWarps);
		}
		mbar_init(done, 1);
		*abort_flag = 0;
		*epi_fail = 0;
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

	// items: column tile major, output tile minor; each CTA a contiguous range
	const long long i0 = static_cast<long long>(blockIdx.x) * p.items / gridDim.x;
	const long long i1 = static_cast<long long>(blockIdx.x + 1) * p.items / gridDim.x;

	if (warp == 0) {
		if (lane == 0) {
			// producer
			asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmap) : "memory");
			unsigned seq = 0;
			bool ok = true;
			for (long long it = i0; ok && it < i1; ++it) {
				const int t = static_cast<int>(it % p.tiles), ct = static_cast<int>(it / p.tiles);
				const int c0 = __ldg(p.chunk_begin + t), nc = __ldg(p.chunk_begin + t + 1) - c0;
				const int kb = __ldg(p.kbase + t);
				for (int c = 0; c < nc; ++c, ++seq) {
					const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
					if (*abort_flag || !mbar_wait(&raw_empty[st], ph ^ 1)) {
						if (!*abort_flag)
							record_failure(2, abort_flag);
						ok = false;
						break;
					}
					unsigned char *stage = sm + st * kStageBytes;
					mbar_arrive_expect_tx(&raw_full[st], kStageBytes);
					tma_load_2d(stage, &tmap, ct * kCols, kb + kKC * c, &raw_full[st]);
					bulk_load(stage + kRawBytes, p.chunk + static_cast<size_t>(c0 + c) * (kABytes / 16), kABytes,
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
			const unsigned xbase = smem_addr(sm + kOffX), sbase = smem_addr(sm);
			unsigned seq = 0, iseq = 0;
			bool ok = true;
			for (long long it = i0; ok && it < i1; ++it, ++iseq) {
				const int t = static_cast<int>(it % p.tiles);
				const int nc = __ldg(p.chunk_begin + t + 1) - __ldg(p.chunk_begin + t);
				const unsigned db = iseq & 1, dph = (iseq >> 1) & 1;
				if (*abort_flag || !mbar_wait(&d_empty[db], dph ^ 1)) {
					if (!*abort_flag)
						record_failure(3, abort_flag);
					break;
				}
				const uint32_t d = tmem + db * kCols;
				for (int c = 0; c < nc; ++c, ++seq) {
					const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
					const unsigned xb = seq & 1, xph = (seq >> 1) & 1;
					if (*abort_flag || !mbar_wait(&x_full[xb], xph) || !mbar_wait(&raw_full[st], ph)) {
						if (!*abort_flag)
							record_failure(3, abort_flag);
						ok = false;
						break;
					}
					tc_fence_after();
					const unsigned xhi = xbase + xb * kXBuf, xlo = xhi + kXOp, ab = sbase + st * kStageBytes + kRawBytes;
#pragma unroll
					for (int s = 0; s < kKC / 8; ++s) {
						const uint64_t da = umma_desc(ab + s * (kABytes / 2), kLboA, kSbo);
						umma_tf32(d, da, umma_desc(xhi + 2 * s * kLboX, kLboX, kSbo), c > 0 || s > 0);
						umma_tf32(d, da, umma_desc(xlo + 2 * s * kLboX, kLboX, kSbo), 1);
					}
					umma_commit(&x_empty[xb]);
					umma_commit(&raw_empty[st]);
				}
				if (!ok)
					break;
				umma_commit(&d_full[db]);
			}
			// nothing of this CTA's may still read shared or tensor memory on return
			umma_commit(done);
			if (!mbar_wait(done, 0))
				record_failure(3, abort_flag);
		}
	} else if (warp < 2 + kEpiWarps) {
		// epilogue: TMEM lanes 32 q .. 32 q + 31 belong to warp q of a warpgroup;
		// quadrants 2 and 3 (remainder rows) hand their rows to quadrants 0 and 1
		const int q = warp & 3;
		const uint32_t tl = tmem + (static_cast<uint32_t>(32 * q) << 16);
		float *xrow = xch + ((q & 1) * 32 + lane) * kXchStride;
		unsigned iseq = 0;
		for (long long it = i0; it < i1; ++it, ++iseq) {
			const int t = static_cast<int>(it % p.tiles), ct = static_cast<int>(it / p.tiles);
			const unsigned db = iseq & 1, dph = (iseq >> 1) & 1;
			// the four warps leave together: each records its own outcome
			// before the barrier and all read the common one after it
			const bool got = __all_sync(0xffffffffu, mbar_wait(&d_full[db], dph)) && !*abort_flag;
			if (!got && lane == 0) {
				*epi_fail = 1;
				record_failure(4, abort_flag);
			}
			epilogue_sync();
			if (*epi_fail)
				break;
			tc_fence_after();
			const int o = t * kOut + 32 * (q & 1) + lane;
			for (int piece = 0; piece < kCols / 32; ++piece) {
				float v[32];
				tmem_ld32(tl + db * kCols + piece * 32, v);
				if (q >= 2) {
#pragma unroll
					for (int j = 0; j < 32; j += 4)
						*reinterpret_cast<float4 *>(xrow + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
				}
				epilogue_sync();
				if (q < 2) {
					const int x0 = ct * kCols + piece * 32;
					if (o < p.dst_dim) {
						float *out = reinterpret_cast<float *>(p.dst + static_cast<ptrdiff_t>(o) * p.dst_stride) + x0;
#pragma unroll
						for (int j = 0; j < 32; j += 4) {
							const float4 r = *reinterpret_cast<const float4 *>(xrow + j);
							const float s0 = v[j] + r.x, s1 = v[j + 1] + r.y, s2 = v[j + 2] + r.z, s3 = v[j + 3] + r.w;
							if (p.dst_aligned && x0 + j + 3 < p.columns) {
								*reinterpret_cast<float4 *>(out + j) = make_float4(s0, s1, s2, s3);
							} else if (x0 + j + 3 < p.columns) {
								out[j] = s0;
								out[j + 1] = s1;
								out[j + 2] = s2;
								out[j + 3] = s3;
							} else {
								if (x0 + j < p.columns)
									out[j] = s0;
								if (x0 + j + 1 < p.columns)
									out[j + 1] = s1;
								if (x0 + j + 2 < p.columns)
									out[j + 2] = s2;
							}
						}
					}
				}
				epilogue_sync();
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&d_empty[db]);
		}
	} else {
		// converters: thread = column of the tile
		const int n = (warp - 2 - kEpiWarps) * 32 + lane;
		unsigned seq = 0;
		bool ok = true;
		for (long long it = i0; ok && it < i1; ++it) {
			const int t = static_cast<int>(it % p.tiles);
			const int nc = __ldg(p.chunk_begin + t + 1) - __ldg(p.chunk_begin + t);
			for (int c = 0; c < nc; ++c, ++seq) {
				const unsigned st = seq % kStages, ph = (seq / kStages) & 1;
				const unsigned xb = seq & 1, xph = (seq >> 1) & 1;
				if (__any_sync(0xffffffffu, *abort_flag) ||
				    !__all_sync(0xffffffffu, mbar_wait(&raw_full[st], ph) && mbar_wait(&x_empty[xb], xph ^ 1))) {
					if (lane == 0 && !*abort_flag)
						record_failure(1, abort_flag);
					ok = false;
					break;
				}
				const unsigned char *stage = sm + st * kStageBytes;
				const float *raw = reinterpret_cast<const float *>(stage);
				unsigned char *xhi = sm + kOffX + xb * kXBuf, *xlo = xhi + kXOp;
				float x[kKC];
#pragma unroll
				for (int k = 0; k < kKC; ++k)
					x[k] = raw[k * kCols + n];
				uint32_t hi[kKC], lo[kKC];
#pragma unroll
				for (int k = 0; k < kKC; ++k)
					split(x[k], hi[k], lo[k]);
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&raw_empty[st]);
#pragma unroll
				for (int kq = 0; kq < kKC / 4; ++kq) {
					const unsigned off = (n >> 3) * kSbo + kq * kLboX + (n & 7) * 16;
					*reinterpret_cast<uint4 *>(xhi + off) =
						make_uint4(hi[4 * kq], hi[4 * kq + 1], hi[4 * kq + 2], hi[4 * kq + 3]);
					*reinterpret_cast<uint4 *>(xlo + off) =
						make_uint4(lo[4 * kq], lo[4 * kq + 1], lo[4 * kq + 2], lo[4 * kq + 3]);
				}
				asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&x_full[xb]);
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

} // namespace

int wide_umma_items(const PassLaunch &l)
{
	return static_cast<int>((l.lines + kCols - 1) / kCols) * l.wide.utiles;
}

cudaError_t launch_wide_umma(const PassLaunch &l, cudaStream_t stream)
{
	const WideTables &w = l.wide;
	if (!w.uchunk || l.horizontal || l.src_stride <= 0 || reinterpret_cast<uintptr_t>(l.src) % 16 || l.src_stride % 16)
		return cudaErrorNotSupported;
	CUtensorMap map;
	if (!encode_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, l.src, l.lines, l.t.input_width,
	                          static_cast<uint64_t>(l.src_stride), kCols, kKC, false))
		return cudaErrorNotSupported;
	UmmaPass p{};
	p.chunk = w.uchunk;
	p.chunk_begin = w.uchunk_begin;
	p.kbase = w.ukbase;
	p.tiles = w.utiles;
	p.items = wide_umma_items(l);
	p.columns = static_cast<int>(l.lines);
	p.dst_dim = static_cast<int>(l.t.rows);
	p.dst = static_cast<char *>(l.dst);
	p.dst_stride = l.dst_stride;
	p.dst_aligned = reinterpret_cast<uintptr_t>(l.dst) % 16 == 0 && l.dst_stride % 16 == 0;
	if (p.items <= 0)
		return cudaSuccess;
	const int grid = std::min(p.items, sm_count_umma());
	const cudaError_t e = cudaFuncSetAttribute(wide_umma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                           static_cast<int>(kSmemBytes));
	if (e != cudaSuccess)
		return e;
	wide_umma_kernel<<<grid, kThreads, kSmemBytes, stream>>>(map, p);
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
