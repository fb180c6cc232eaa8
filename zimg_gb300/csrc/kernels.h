// Launch interface between the host planner and the CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace zg {

// Device-resident tap tables of one pass (the GPU copy of a FilterTable).
//   left[i]            first input sample of output i
//   f32[i*width + k]   float taps
//   i16[i*width + k]   signed 1.14 taps
//   bias[i]            -32768 * sum_k i16[i*width+k] (mod 2^32): folds zimg's
//                      "x - 32768" unpacking (resize_impl.cpp:31-34) into one
//                      constant so the inner loop is a plain multiply-add.
struct PassTables {
	const unsigned *left;
	const float *f32;
	const int16_t *i16;
	const int32_t *bias;
	unsigned width;        // taps per output
	unsigned rows;         // outputs along the filtered axis
	unsigned input_width;  // inputs along the filtered axis
	// FP32 passes of at least kDenseTaps taps, on CUDA cores: outputs in groups
	// of dense_rows(horizontal) (8 vertically, 4 horizontally); group g's taps
	// as a dense block over the inputs dbase[g] + u, u < dspan[g] (exact zeros
	// outside each output's band), so that an input is loaded once per group:
	// vertical passes dense[(g * dstride + u) * 8 + r], horizontal ones
	// dense[(u * groups + g) * 4 + r] (a warp's 32 groups side by side);
	// dwin: the widest input window of 32 consecutive horizontal groups
	const float *dense;
	const unsigned *dbase;
	const unsigned *dspan;
	unsigned dstride;
	unsigned dwin;
};

constexpr unsigned kDenseTaps = 32;
__host__ __device__ constexpr unsigned dense_rows(bool horizontal)
{
	return horizontal ? 4u : 8u;
}

enum class Sample { U16, F32 };

// Band fragments of one FP32 pass for the tensor-core kernel (wide_kernel.cu).
// Outputs are taken 8 at a time ("output groups"); group g covers outputs
// 8g..8g+7 and the inputs [kbase[g], kbase[g] + 8 * ksteps), over which its
// taps form a dense 8 x (8 * ksteps) block (zero outside each output's band).
// frag[(g * ksteps + s) * 32 + lane] holds the mma.m16n8k8 B fragment of
// k-step s for that lane, both tf32 halves of each f32 tap:
//   {b0 high, b1 high, b0 low, b1 low},  b0 = tap(8g + lane/4, kbase + 8s + lane%4),
//   b1 = the same 4 inputs further (horizontal passes: b0 at input
//   kbase + 8s + 2 (lane%4), b1 the next input, kbase even); high = tap
//   rounded to tf32, low = (tap - high) rounded to tf32.
struct WideTables {
	const uint4 *frag;     // null: the pass runs on the CUDA cores
	const int *kbase;
	int groups;
	int ksteps;
	// The tcgen05 form of vertical passes (wide_umma.cu): tiles of 64
	// outputs, bands cut into chunks of 16 input rows. Null uchunk: only the
	// mma.sync form exists (horizontal passes).
	const uint4 *uchunk;      // per chunk: two 8-row blocks of [64 hi taps; 64 lo taps], UMMA K-major layout (8 KB)
	const int *uchunk_begin;  // per tile: index of its first chunk; [utiles] = number of chunks
	const int *ukbase;        // per tile: first input row of its band
	int utiles;
	int umax_taps;            // widest band of one output (taps)
};

// One pass over a whole plane. For a horizontal pass the plane has
// `lines` rows of input_width samples -> rows outputs each; for a vertical
// pass it has `lines` columns, input_width rows -> rows rows.
struct PassLaunch {
	PassTables t;
	bool horizontal;
	Sample sample;
	int32_t pixel_max;     // (1 << depth) - 1 for U16
	unsigned lines;        // height (H) or width (V) of the plane
	const void *src;
	ptrdiff_t src_stride;  // bytes
	void *dst;
	ptrdiff_t dst_stride;  // bytes
	WideTables wide;       // FP32 passes on the tensor cores when wide.frag is set
};

// Host side of WideTables: fragments and group bases of a pass with `rows`
// outputs of `width` taps (f32[i * width + k] applies to input left[i] + k).
void build_wide_tables(const float *f32, const unsigned *left, unsigned width, unsigned rows, bool perm_k,
                       std::vector<uint4> *frag, std::vector<int> *kbase, int *ksteps);

cudaError_t launch_wide(const PassLaunch &l, cudaStream_t stream);

// Host side of the tcgen05 form of a vertical pass: per tile of 64 outputs
// its band base and its chunks' tap blocks.
void build_umma_tables(const float *f32, const unsigned *left, unsigned width, unsigned rows,
                       std::vector<uint4> *chunks, std::vector<int> *chunk_begin, std::vector<int> *kbase);
// Work items of a vertical pass on the tcgen05 form (tiles of 256 columns x
// 64 outputs).
int wide_umma_items(const PassLaunch &l);
// The vertical pass on the tcgen05 kernel when the plane allows it (16-byte
// aligned source, positive stride): cudaErrorNotSupported otherwise, nothing
// launched.
cudaError_t launch_wide_umma(const PassLaunch &l, cudaStream_t stream);
// The forms of the wide passes enqueued by this host thread since the last
// reset (bit 0 mma.sync, bit 1 tcgen05).
int wide_forms_used(bool reset);
// Nonzero when a pipeline wait of the tcgen05 kernel ran out (optionally reset).
int wide_umma_pipeline_error(bool reset);

// Planes that a batch copies unchanged (conversions with no pass,
// resize.cpp:43-47): one launch for all of them. Each plane is split into
// `unit`-byte chunks (16 when both planes and strides allow it, else the
// sample size); chunk_begin is the plane's first chunk in the launch.
struct PlaneCopy {
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;
	unsigned row_bytes;
	unsigned rows;
	unsigned unit;
	unsigned chunks_per_row;
	unsigned long long chunk_begin;
};

cudaError_t launch_plane_copies(const PlaneCopy *table, int n, unsigned long long total_chunks, cudaStream_t stream);

cudaError_t launch_pass(const PassLaunch &l, cudaStream_t stream);

} // namespace zg
