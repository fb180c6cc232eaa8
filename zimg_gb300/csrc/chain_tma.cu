// Host side of the TMA-pipelined chained kernel (chain_tma_kernel.cuh):
// shared-memory layout, source tensor maps, launch, instantiations.
#include "chain_tma_kernel.cuh"
#include "fused.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <mutex>

namespace zg {

namespace {

constexpr size_t kTmaSmemMax = 110 * 1024;  // two CTAs per SM
constexpr int kKVMax = 3;
constexpr int kKHMax = 4;
constexpr int kMaxBoxW = 256;               // tensor-copy box limit per dimension
constexpr int kAlignSlack = 128;            // the kernel aligns its shared-memory base to 128 bytes

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's tensor-map encoder, looked up once through the runtime.
EncodeTiled encoder()
{
	static EncodeTiled fn = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q{};
		if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<EncodeTiled>(p);
	});
	return fn;
}

template <bool HF, int KV, int KH>
const void *tma_ptr()
{
	return reinterpret_cast<const void *>(&chain_detail::chain_tma_kernel<HF, KV, KH>);
}

template <bool HF, int KV>
const void *tma_ptr_kh(int kh)
{
	switch (kh) {
	case 1: return tma_ptr<HF, KV, 1>();
	case 2: return tma_ptr<HF, KV, 2>();
	case 3: return tma_ptr<HF, KV, 3>();
	default: return tma_ptr<HF, KV, 4>();
	}
}

template <bool HF>
const void *tma_ptr_kv(int kv, int kh)
{
	return kv == 1 ? tma_ptr_kh<HF, 1>(kh) : (kv == 2 ? tma_ptr_kh<HF, 2>(kh) : tma_ptr_kh<HF, 3>(kh));
}

int tma_threads(int variant)
{
	return chain_detail::tma_threads(variant - 200 >= kKVMax * kKHMax);
}

} // namespace

const void *chain_tma_kernel_ptr(int variant)
{
	const int v = variant - 200;
	const int per = kKVMax * kKHMax;
	const bool hf = v >= per;
	const int kv = (v % per) / kKHMax + 1, kh = v % kKHMax + 1;
	return hf ? tma_ptr_kv<true>(kv, kh) : tma_ptr_kv<false>(kv, kh);
}

bool chain_tma_enabled()
{
	// the default where the source planes admit a tensor map; ZG_CHAIN_TMA=0
	// keeps the cp.async form
	static const bool on = [] {
		const char *e = std::getenv("ZG_CHAIN_TMA");
		return !(e && e[0] == '0');
	}();
	return on;
}

bool chain_tma_layout(const FusedPlan *const *plans, int n, SmemLayout *out)
{
	int max_pxa = 0, in = 1, groups = 1, depth = 1, kv = 1, tiles = 1;
	for (int i = 0; i < n; ++i) {
		const FusedPlan &p = *plans[i];
		if (!p.chain)
			return false;
		max_pxa = std::max(max_pxa, p.max_pxa);
		in = std::max(in, p.job.in_rows);
		groups = std::max(groups, p.job.groups);
		depth = std::max(depth, p.depth);
		kv = std::max(kv, p.job.vs);
		tiles = std::max(tiles, chain_detail::tiles_per_warp(p.job.vs, p.job.hw));
	}
	auto a16 = [](size_t x) { return static_cast<int>((x + 15) / 16 * 16); };
	auto pow2 = [](int x) {
		int p = 1;
		while (p < x)
			p *= 2;
		return p;
	};
	SmemLayout L{};
	// box rows of 16 mod 32 bytes (8 mod 16 samples) covering the widest
	// window: 4-byte fragment loads of 8 lines x 4 pairs hit 32 different
	// banks, the 8 rows of an ldmatrix phase 8 different 16-byte bank groups
	L.pitch = std::max(8, (max_pxa - 8 + 15) / 16 * 16 + 8);
	if (L.pitch > kMaxBoxW)
		return false;
	L.stage_rows = 1;
	L.seg_groups = groups;
	L.step_groups = 1;
	L.depth = depth;
	// ring: 2^n blocks, as many as cover the plan's lines in flight, but no
	// fewer than a window's blocks plus one (a window of 16 KV lines touches
	// KV + 1 blocks); stages: the plan's depth + 2, no fewer than 3. The
	// largest ring, then the most stages, that fit the shared-memory budget.
	const int nb_want = pow2((in + 2 * (chain_detail::kBlockLines - 1)) / chain_detail::kBlockLines + 1);
	const int nb_min = pow2(kv + 2);
	for (int nb = nb_want; nb >= nb_min; nb /= 2) {
		for (int ns = depth + 2; ns >= 3; --ns) {
			L.in_rows = nb * chain_detail::kBlockLines;
			L.ring_rows = ns;  // pipeline stages
			int off = 0;
			L.in_off = off;
			off += a16(static_cast<size_t>(L.in_rows) * L.pitch * 2);
			L.vcoef_off = off;
			off += a16(static_cast<size_t>(L.ring_rows) * kv * 2 * 32 * 16);
			L.tile_off = off;
			L.tile_pitch = chain_detail::kStageBytes / 2;
			off += a16(static_cast<size_t>(chain_detail::kWsWarps) * tiles * chain_detail::kTileStage);
			L.vbase_off = off;
			off += a16(static_cast<size_t>(groups) * 4);
			L.stage_off = off;  // full and empty mbarriers
			off += a16(static_cast<size_t>(L.ring_rows) * 2 * 8);
			L.ring_off = L.i_off = L.htaps_off = L.hleft_off = off;
			L.total_bytes = off + kAlignSlack;
			if (static_cast<size_t>(L.total_bytes) <= kTmaSmemMax) {
				*out = L;
				return true;
			}
		}
	}
	return false;
}

bool encode_tensor_map_2d(CUtensorMap *map, CUtensorMapDataType type, const void *base, uint64_t width,
                          uint64_t height, uint64_t stride, uint32_t box_w, uint32_t box_h, bool swizzle128)
{
	EncodeTiled fn = encoder();
	if (!fn || !base || reinterpret_cast<uintptr_t>(base) % 16 || stride % 16 || !width || !height)
		return false;
	const cuuint64_t dims[2] = { width, height };
	const cuuint64_t strides[1] = { stride };
	const cuuint32_t box[2] = { box_w, box_h };
	const cuuint32_t estr[2] = { 1, 1 };
	return fn(map, type, 2, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
	          swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
	          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool chain_tma_source_map(CUtensorMap *map, const FusedJob &j, const SmemLayout &L)
{
	const uintptr_t a = reinterpret_cast<uintptr_t>(j.src);
	if (!j.src || a % 16 || j.src_stride <= 0 || j.src_stride % 16 || j.src_w < 1 || j.src_h < 1)
		return false;
	if (L.pitch > kMaxBoxW || (L.pitch * 2) % 16)
		return false;
	EncodeTiled fn = encoder();
	if (!fn)
		return false;
	const cuuint64_t dims[2] = { static_cast<cuuint64_t>(j.src_w), static_cast<cuuint64_t>(j.src_h) };
	const cuuint64_t strides[1] = { static_cast<cuuint64_t>(j.src_stride) };
	const cuuint32_t box[2] = { static_cast<cuuint32_t>(L.pitch), static_cast<cuuint32_t>(chain_detail::kBlockLines) };
	const cuuint32_t estr[2] = { 1, 1 };
	return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(j.src), dims, strides, box, estr,
	          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
	          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int chain_tma_grid_size(int variant, size_t smem_bytes)
{
	int dev = 0, sms = 0, per_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const void *k = chain_tma_kernel_ptr(variant);
	cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTmaSmemMax));
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, tma_threads(variant), smem_bytes) != cudaSuccess ||
	    per_sm < 1)
		per_sm = 1;
	return std::max(1, sms) * per_sm;
}

cudaError_t launch_chain_tma(int variant, const FusedJob *jobs, int num_jobs, int total_items, const int *ranges,
                             const SmemLayout &L, int grid, const FusedJob &single, const CUtensorMap *single_map,
                             cudaStream_t stream)
{
	if (static_cast<size_t>(L.total_bytes) > kTmaSmemMax || (!jobs && !single_map))
		return cudaErrorInvalidValue;
	const void *k = chain_tma_kernel_ptr(variant);
	cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTmaSmemMax));
	if (e != cudaSuccess)
		return e;
	FusedJob one = single;
	SmemLayout layout = L;
	CUtensorMap map{};
	if (single_map)
		map = *single_map;
	void *args[] = { &jobs, &num_jobs, &total_items, &ranges, &one, &layout, &map };
	if (!ranges)
		grid = std::max(1, std::min(grid, total_items));
	return cudaLaunchKernel(k, dim3(grid), dim3(tma_threads(variant)), args, static_cast<size_t>(L.total_bytes),
	                        stream);
}

std::vector<int> chain_tma_lockstep_ranges(int total_items, int groups, int grid)
{
	std::vector<int> r;
	if (groups <= 0 || grid <= 0 || total_items % groups || total_items / groups < grid)
		return r;
	const long long lead = static_cast<long long>(grid) * groups;
	const long long rest = total_items - lead;
	r.resize(4 * static_cast<size_t>(grid));
	for (int b = 0; b < grid; ++b) {
		r[4 * b] = b * groups;
		r[4 * b + 1] = (b + 1) * groups;
		r[4 * b + 2] = static_cast<int>(lead + rest * b / grid);
		r[4 * b + 3] = static_cast<int>(lead + rest * (b + 1) / grid);
	}
	return r;
}

int chain_mixed_copy_variant()
{
	return chain_detail::kCopyVariant;
}

int chain_mixed_grid_size(size_t smem_bytes)
{
	int dev = 0, sms = 0, per_sm = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const void *k = reinterpret_cast<const void *>(&chain_detail::chain_mixed_kernel);
	cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTmaSmemMax));
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, chain_detail::tma_threads(true), smem_bytes) !=
	        cudaSuccess ||
	    per_sm < 1)
		per_sm = 1;
	return std::max(1, sms) * per_sm;
}

cudaError_t launch_chain_mixed(const FusedJob *jobs, int num_jobs, const WorkChunks &chunks, const SmemLayout &L,
                               int grid, cudaStream_t stream)
{
	if (static_cast<size_t>(L.total_bytes) > kTmaSmemMax || !jobs || !chunks.bounds || !chunks.sched ||
	    chunks.num < 1 || grid < 1)
		return cudaErrorInvalidValue;
	const void *k = reinterpret_cast<const void *>(&chain_detail::chain_mixed_kernel);
	cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTmaSmemMax));
	if (e != cudaSuccess)
		return e;
	SmemLayout layout = L;
	WorkChunks C = chunks;
	grid = std::min(grid, C.num);
	void *args[] = { &jobs, &num_jobs, &C, &layout };
	return cudaLaunchKernel(k, dim3(grid), dim3(chain_detail::tma_threads(true)), args,
	                        static_cast<size_t>(L.total_bytes), stream);
}

int chain_tma_set_fault(int drop_group, unsigned long long wait_ns)
{
	if (cudaMemcpyToSymbol(chain_detail::g_chain_drop_group, &drop_group, sizeof(drop_group)) != cudaSuccess ||
	    cudaMemcpyToSymbol(chain_detail::g_chain_wait_ns, &wait_ns, sizeof(wait_ns)) != cudaSuccess)
		return -1;
	return 0;
}

int chain_tma_pipeline_error(bool reset)
{
	int v = 0;
	if (cudaMemcpyFromSymbol(&v, chain_detail::g_chain_pipeline_error, sizeof(v)) != cudaSuccess)
		return -1;
	if (reset && v) {
		const int zero = 0;
		cudaMemcpyToSymbol(chain_detail::g_chain_pipeline_error, &zero, sizeof(zero));
	}
	return v;
}

} // namespace zg
