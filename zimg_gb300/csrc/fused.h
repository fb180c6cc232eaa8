// Fused two-pass resize: both passes of a conversion in one kernel, one output
// tile per CTA iteration, the intermediate kept in shared memory.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "filter_plan.h"

namespace zg {

// Arithmetic of a fused job.
//   F32:      float samples, taps applied in zimg's order with one fused
//             multiply-add each; float intermediate.
//   U16_EXACT: u16 samples computed in float on exact integers: samples are
//             re-centred (v - 2^(depth-1)), taps are zimg's int16 taps, and the
//             planner has proved that every partial sum stays below 2^24, so
//             each multiply-add is exact and the result equals zimg's int32
//             arithmetic bit for bit (resize_impl.cpp:31-59,78-95).
enum class FusedKind : int { F32 = 0, U16_EXACT = 1 };

// Compile-time buckets. V passes use groups of kGroup outputs whose taps are
// laid out densely over a window of S input lines (S = 8, 12, 16 or 24);
// H passes use per-output taps padded with zeros to W (4, 8, 12, 16).
constexpr int kGroup = 4;
constexpr int kTileThreads = 256;

// One fused job as the kernel sees it (device-resident table entry).
struct FusedJob {
	// planes (filled from the batch's io table)
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;

	// geometry
	int h_first;            // 1: H then V; 0: V then H
	int kind;               // FusedKind
	int src_w, src_h, dst_w, dst_h;
	int tile_h, tile_w;     // output tile
	int tiles_x, tiles_y;
	int tile_begin;         // first global tile index of this job

	// H pass: taps padded to hw per output column, left[] per output column
	const float *h_taps;    // [dst_w][hw]
	const int *h_left;      // [dst_w]
	int hw;

	// V pass: dense groups of kGroup output rows over vs input lines
	const float *v_dense;   // [groups][kGroup][vs]
	const int *v_base;      // [groups]
	int vs;

	// per tile row / tile column: input window of the patch
	const int *win_row;     // [tiles_y][2]  rows [lo, hi) of the source
	const int *win_col;     // [tiles_x][2]  cols [lo, hi) of the source (lo aligned down)

	// u16 exact arithmetic
	float magic;            // 1.5*2^23 + offset
	float pixel_max;
	float offset;           // 2^(depth-1)
	int vec_ok;             // planes and strides 16-byte aligned: vector loads and stores
};

// Shared-memory layout of one launch (the maximum over its jobs): two
// prefetch buffers, each holding a patch and the tile's tap tables, then the
// converted-float patch (u16 only) and the intermediate.
struct SmemLayout {
	int buf_bytes;
	int vcoef_off, htaps_off, hleft_off, vbase_off;  // within a buffer
	int pf_off;                                      // from the start
	int i_off;
	int total_bytes;
};

// Fill the plane pointers of a job and its alignment flag.
void fused_set_io(FusedJob &j, const void *src, ptrdiff_t src_stride, void *dst, ptrdiff_t dst_stride);

// Host-side plan of one fused job: device tables plus a FusedJob template
// (without plane pointers).
struct FusedPlan {
	FusedJob job{};
	size_t smem_bytes = 0;   // dynamic shared memory this job needs
	int max_py = 0, max_pitch = 0;  // largest patch (rows, elements per row)
	int variant = 0;         // kernel instantiation index
	std::vector<unsigned char> blob;  // host copy of the tables, uploaded by the owner
	size_t off_h_taps = 0, off_h_left = 0, off_v_dense = 0, off_v_base = 0, off_win_row = 0, off_win_col = 0;
};

// Try to build a fused plan for a two-pass conversion. Returns false (and
// leaves the conversion to the two-pass kernels) when the job is not fusable:
// taps too wide for the buckets, patch larger than the shared-memory budget,
// or u16 sums that cannot be proved exact in float.
bool plan_fused(const FilterTable &first, const FilterTable &second, bool h_first, bool u16, unsigned depth,
                unsigned src_w, unsigned src_h, unsigned dst_w, unsigned dst_h, FusedPlan *out);

// Point the job's table pointers at `device_blob` (the uploaded copy of blob).
void fused_bind(FusedPlan &p, const void *device_blob);

// Launch all tiles of `jobs` (a device array of num_jobs FusedJob, all of the
// same variant) as one persistent grid; with jobs == nullptr, run `single`
// (passed by value as a kernel parameter).
cudaError_t launch_fused(int variant, const FusedJob *jobs, int num_jobs, int total_tiles, const SmemLayout &L,
                         int grid, const FusedJob &single, cudaStream_t stream);

// Shared-memory layout that covers every plan in `plans` (all one variant).
SmemLayout fused_layout(const FusedPlan *const *plans, int n);

// Largest dynamic shared memory any variant may use, and the CTA count per SM
// the launcher targets.
size_t fused_max_smem();
int fused_grid_size(int variant, size_t smem_bytes);

} // namespace zg
