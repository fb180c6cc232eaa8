// Depth conversion kernel interface (depth_kernel.cu) and zimg's choice of
// conversion (depth.cpp:43-66, quantize.h:19-45), shared by the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace zg {

struct DepthLaunch {
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;
	int width, height;
	float scale, offset;  // mode 2 and 3: x * scale + offset
	float vmax;           // mode 3: 2^depth - 1
	unsigned shift;       // mode 1
	unsigned seq;         // mode 3: plane index (dither table variant)
	int dither;           // mode 3: 0 none, 1 ordered, 2 random
	int vec_in, vec_out;  // planes aligned for 8-sample vector loads / stores
};

// in_type / out_type: 0 BYTE, 1 WORD, 2 HALF, 3 FLOAT; mode 1 left shift,
// 2 to FLOAT or HALF, 3 dither to integer.
cudaError_t launch_depth(int in_type, int out_type, int mode, const DepthLaunch &L, cudaStream_t stream);

// Error diffusion (ed_kernel.cu). One thread block per plane; in a block,
// warp w takes bands of 32 lines b = w, w + warps, ..., one line per lane.
// Line r of a band processes column c at band step c + 3r, and band b starts
// `spacing` steps after band b - 1, so every sample comes after the three
// samples of the line above that it reads (columns c - 1 .. c + 1) and after
// its left neighbour.
constexpr int kEdMaxPlanes = 4;
constexpr int kEdChunk = 16;   // band steps between block-wide barriers
constexpr int kEdLag = 3;      // columns a line runs behind the line above
constexpr int kEdPitch = 17;   // words per lane in the staging tiles (conflict-free)

struct EdPlane {
	const void *src;
	ptrdiff_t src_stride;
	void *dst;
	ptrdiff_t dst_stride;
	int width, height;
	float scale, offset, vmax;
	int bands;    // ceil(height / 32)
	int spacing;  // steps between band starts, a multiple of kEdChunk
	int cycle;    // steps between the bands of one warp (no second band: 2^30)
	int steps;    // steps until the last band ends, a multiple of kEdChunk
};

struct EdLaunch {
	EdPlane planes[kEdMaxPlanes];
	int num_planes;
	int in_type, out_type;  // as launch_depth; out BYTE or WORD
	int warps;              // warps per block (bands in flight)
	int ring;               // floats in each warp's hand-off ring, a power of 2
};

// Shape of one plane's launch for `warps` warps per block: fills spacing,
// steps and the ring it needs; false if no shape fits the shared memory.
bool ed_shape(EdPlane &p, int warps, int *ring);
// Warps per block for a plane of this size (a cost model of the wavefront).
int ed_choose_warps(int width, int height);
// Dynamic shared memory of a launch.
size_t ed_smem_bytes(int warps, int ring);
cudaError_t launch_error_diffusion(const EdLaunch &L, cudaStream_t stream);

} // namespace zg

struct zg_depth;

namespace zg {

// The error-diffusion plane of a depth conversion object (its size, scale,
// offset and range; pointers unset) and its pixel types; false when the
// conversion does not diffuse errors.
bool depth_ed_plane(const ::zg_depth *d, EdPlane *plane, int *in_type, int *out_type);

} // namespace zg
