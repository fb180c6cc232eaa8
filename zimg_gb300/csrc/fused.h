// Fused two-pass resize: both passes of a conversion in one kernel. Each CTA
// owns a strip of 128 output columns and streams the source rows of a row
// segment through a ring of lines in shared memory, so every source line is
// read from HBM and filtered once and the intermediate never reaches HBM.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "filter_plan.h"
#include "work_chunks.h"

namespace zg {

// Arithmetic of a fused job.
//   F32:       float samples, taps applied in zimg's order with one fused
//              multiply-add each; float intermediate.
//   U16_EXACT: u16 samples computed in float on exact integers: samples are
//              re-centred (v - 2^(depth-1)), taps are zimg's int16 taps, and the
//              planner has proved that every partial sum stays below 2^24, so
//              each multiply-add is exact and the result equals zimg's int32
//              arithmetic bit for bit (resize_impl.cpp:31-59,78-95).
//   U16_INT:   u16 samples where that proof fails (deeper samples: 12-bit,
//              16-bit): zimg's own int32 arithmetic, samples centred by 32768
//              (unpack_pixel_u16), 8192 + sum(tap * sample) in int32, then
//              (sum >> 14) + 32768 clamped to the depth (pack_pixel_u16);
//              planned where |taps| * 2^15 + 8192 stays below 2^31.
enum class FusedKind : int { F32 = 0, U16_EXACT = 1, U16_INT = 2 };

// Vertical taps come in groups of group_rows() output rows laid out densely over a
// window of VS input lines (VS = 8, 12, 16 or 24); horizontal taps per output
// column are padded with zeros to HW (6, 8 or 16).
// Rows per vertical group: 4 for H-first conversions (upscales: one line load
// feeds 4 rows), 2 for V-first ones (downscales: narrower dense windows).
__host__ __device__ constexpr int group_rows(bool h_first)
{
	return h_first ? 4 : 2;
}
constexpr int kStripW = 128;      // output columns per strip
constexpr int kStreamThreads = 128;

// One fused job as the kernel sees it (device-resident table entry).
struct FusedJob {
	// planes (filled from the caller's io)
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;

	int h_first;            // 1: H then V; 0: V then H
	int kind;               // FusedKind
	int src_w, src_h, dst_w, dst_h;

	// work items: strips x row segments
	int strips;             // ceil(dst_w / strip_w)
	int strip_w;            // output columns per strip (kStripW for the CUDA-core kernel)
	int segments;           // row segments per strip (chained kernel: one per group)
	int seg_groups;         // vertical groups per segment (last may be shorter)
	int groups;             // vertical groups of the plane (ceil(dst_h / group_rows))
	int step_groups;        // vertical groups per streaming step
	int item_begin;         // first global item index of this job

	// rings (lines), powers of two
	int ring_rows;          // V-first: source lines; H-first: intermediate lines
	int depth;              // steps of source lines in flight (tensor-core kernel)
	int in_rows;            // H-first: source lines staged for the H pass

	// H pass: taps padded to hw per output column, left[] per output column
	const float *h_taps;    // [dst_w][hw]
	const int *h_left;      // [dst_w]
	int hw;
	// V pass: dense groups of group_rows output rows over vs input lines
	const float *v_dense;   // [groups][vs][group_rows]
	const int *v_base;      // [groups] first input line of each group (non-decreasing)
	int vs;

	const int *win_col;     // [strips][2] source columns [lo, hi) (lo aligned down)

	// u16 exact arithmetic
	float magic;            // 1.5*2^23 + offset
	float pixel_max;
	float offset;           // 2^(depth-1)
	int vec_ok;             // planes and strides 16-byte aligned: vector loads and stores
	const void *tmap;       // TMA-pipelined chained kernel: the source plane's tensor map (device memory)
	int variant;            // chained kernel's variant - 200 ((H first, KV, KH)); mixed launches dispatch on it
};

// Guided work chunks of a persistent launch (work_chunks.cuh): chunk m is
// the work units [bounds[m], bounds[m + 1]) (device memory, strictly
// increasing, num chunks); CTAs take chunks from the counter sched[0] in the
// order they ask. sched (two words in device memory) is zero before a launch
// and left zero after it; launches that may overlap need their own. With
// sched == nullptr a launch splits its units statically.
struct WorkChunks {
	const int *bounds = nullptr;
	int num = 0;
	unsigned *sched = nullptr;
};

// Shared-memory layout of one launch (the maximum over its jobs).
struct SmemLayout {
	int pitch;              // elements per ring line (largest strip patch + pad)
	int ring_off;           // float ring (V-first source lines / H-first intermediate lines)
	int stage_off;          // raw staging lines (u16 samples before conversion; H-first source lines)
	int in_off;             // H-first: float source lines for the H pass
	int i_off;              // V-first: intermediate lines of one step
	int htaps_off, hleft_off;
	int vcoef_off;          // two buffers of one step's vertical tap groups
	int vbase_off;          // one segment's group bases
	int total_bytes;
	int ring_rows, in_rows, stage_rows, seg_groups, step_groups;
	int depth;              // steps of lines in flight ahead of the computing step
	int tile_off, tile_pitch;  // tensor-core kernel: staged output rows (packed u16)
};

// Host-side plan of one fused job: device tables plus a FusedJob template.
struct FusedPlan {
	FusedJob job{};
	int variant = 0;         // kernel instantiation index
	int max_pxa = 0;         // widest strip patch (elements)
	int stage_rows = 1;      // u16 raw staging lines
	int depth = 1;           // prefetch depth in steps
	bool mma = false;        // tensor-core variant (mma_kernel.cuh or chain_kernel.cuh)
	bool chain = false;      // tensor-core variant with the passes chained in registers (chain_kernel.cuh)
	float reuse_frac = 0;    // chained H-first plans: share of groups that reuse the previous group's products
	std::vector<unsigned char> blob;  // host copy of the tables, uploaded by the owner
	size_t off_h_taps = 0, off_h_left = 0, off_v_dense = 0, off_v_base = 0, off_win_col = 0;
};

// Fill the plane pointers of a job and its alignment flag.
void fused_set_io(FusedJob &j, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride);

// Try to build a fused plan for a two-pass conversion. Returns false (and
// leaves the conversion to the two-pass kernels) when the job is not fusable:
// taps too wide for the buckets, window tables that are not monotonic, rings
// larger than the shared-memory budget, or u16 sums that cannot be proved
// exact in float.
bool plan_fused(const FilterTable &first, const FilterTable &second, bool h_first, bool u16, unsigned depth,
                unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out);

// Split each plan's strips into row segments so that about
// `num_items_target` work items exist across `plans` in total.
void fused_segment(FusedPlan *const *plans, int n, int num_items_target);

// Point the job's table pointers at `device_blob` (the uploaded copy of blob).
void fused_bind(FusedPlan &p, const void *device_blob);

// Shared-memory layout that covers every plan in `plans` (all one variant).
SmemLayout fused_layout(const FusedPlan *const *plans, int n);

// Launch all items of `jobs` (a device array of num_jobs FusedJob, all of the
// same variant) as one persistent grid; with jobs == nullptr, run `single`
// (passed by value as a kernel parameter).
cudaError_t launch_fused(int variant, const FusedJob *jobs, int num_jobs, int total_items, const SmemLayout &L,
                         int grid, const FusedJob &single, cudaStream_t stream, const WorkChunks &chunks = {});
// Whether launch_fused takes guided chunks for this variant (the CUDA-core
// streaming kernel does; the tensor-core forms launched through it split
// their units statically).
bool fused_takes_chunks(int variant);

size_t fused_max_smem();
int fused_grid_size(int variant, size_t smem_bytes);
int fused_items(const FusedJob &j);

// Tensor-core u16 variant (exact, depth <= 12): same job table and streaming
// structure; tap tables are mma fragments (h_taps/v_dense) and column-group
// bases (h_left). Variants are numbered from 100.
bool plan_mma(const FilterTable &first, const FilterTable &second, bool h_first, unsigned depth, unsigned src_w,
              unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out);
SmemLayout mma_layout(const FusedPlan *const *plans, int n);
cudaError_t launch_mma(int variant, const FusedJob *jobs, int num_jobs, int total_items, const SmemLayout &L, int grid,
                       const FusedJob &single, cudaStream_t stream);
const void *mma_kernel_ptr(int variant);
int mma_threads();

// Chained tensor-core u16 kernel (chain_kernel.cuh): variants 200+. Same
// exactness certificate as plan_mma; 16-column tiles per warp, windows of up
// to 3 x 16 lines and 4 x 16 columns.
bool plan_chain(const FilterTable &first, const FilterTable &second, bool h_first, unsigned depth, unsigned src_w,
                unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out);
SmemLayout chain_layout(const FusedPlan *const *plans, int n);
const void *chain_kernel_ptr(int variant);
int chain_threads(int variant);
cudaError_t launch_chain(int variant, const FusedJob *jobs, int num_jobs, int total_items, const SmemLayout &L, int grid,
                         const FusedJob &single, cudaStream_t stream);
// The same kernel with source lines and tap fragments brought in by tensor
// copies on an mbarrier pipeline (chain_tma_kernel.cuh). Usable when the
// layout fits (box width <= 256) and the source plane has a tensor map
// (16-byte aligned base and stride).
bool chain_tma_enabled();  // false when the environment sets ZG_CHAIN_TMA=0
bool chain_tma_layout(const FusedPlan *const *plans, int n, SmemLayout *out);
bool chain_tma_source_map(CUtensorMap *map, const FusedJob &j, const SmemLayout &L);
int chain_tma_grid_size(int variant, size_t smem_bytes);
// ranges: null (each CTA an equal contiguous range of the units), or 4 ints
// per CTA of `grid`, two unit ranges each CTA runs in order
// (chain_tma_lockstep_ranges).
cudaError_t launch_chain_tma(int variant, const FusedJob *jobs, int num_jobs, int total_items, const int *ranges,
                             const SmemLayout &L, int grid, const FusedJob &single, const CUtensorMap *single_map,
                             cudaStream_t stream);
// Per-CTA unit ranges for `grid` CTAs over jobs of `groups` units per strip
// and `total_items` units: CTA b first the whole strip b, then an equal share
// of the strips beyond the first `grid`. Empty when there are fewer strips
// than CTAs (equal ranges then).
std::vector<int> chain_tma_lockstep_ranges(int total_items, int groups, int grid);
// Nonzero when a pipeline wait of that kernel ran out (optionally reset).
int chain_tma_pipeline_error(bool reset);
// One launch over a mixed batch (chained jobs of any variant, each FusedJob's
// `variant`, and identity copies, variant chain_mixed_copy_variant(), src_w
// = row bytes, groups = 16-row bands, strips = 1), its units in guided
// chunks (required). L covers every chained job.
int chain_mixed_copy_variant();
int chain_mixed_grid_size(size_t smem_bytes);
cudaError_t launch_chain_mixed(const FusedJob *jobs, int num_jobs, const WorkChunks &chunks, const SmemLayout &L,
                               int grid, cudaStream_t stream);
// Test hook: CTA 0's producer skips group drop_group (-1: none) without
// arming its stage; waits give up after wait_ns (0: the default 0.25 s).
int chain_tma_set_fault(int drop_group, unsigned long long wait_ns);
// A 2-D tensor map (zero fill outside the plane) over a plane of width x
// height elements, `stride` bytes per line; swizzle128: boxes land in shared
// memory with the 128-byte swizzle (16-byte chunk c of box line r at chunk
// c ^ (r % 8); box lines of 128 bytes, destination 1024-byte aligned). False
// when the CUDA driver's tensor-map encoder refuses it or base / stride are
// not 16-byte aligned.
bool encode_tensor_map_2d(CUtensorMap *map, CUtensorMapDataType type, const void *base, uint64_t width,
                          uint64_t height, uint64_t stride, uint32_t box_w, uint32_t box_h, bool swizzle128 = false);
// Work items that fill the current device once (SMs x resident CTAs).
int fused_wave_items();

} // namespace zg
