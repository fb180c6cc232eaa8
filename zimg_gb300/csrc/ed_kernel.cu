// Floyd-Steinberg error diffusion of whole planes to BYTE or WORD (zimg's
// ErrorDiffusion, src/zimg/depth/dither.cpp:59-85 per line and 291-345 over
// the plane), equal bit for bit to zimg's C path.
//
// The recurrence is serial along a line (each sample takes the error of its
// left neighbour) and across lines (the three samples above it, columns
// c - 1 .. c + 1). Lines therefore run as a wavefront: one lane per line,
// 32 lines to a warp ("band"), line r of a band at column c on band step
// c + 3r. A lane needs the line above's error at column c + 1 two steps after
// that lane made it, so the value crosses lanes by shuffle off the critical
// path, which is the left neighbour's error (ten dependent float operations
// a sample). Band b starts `spacing` steps after band b - 1; the last line of
// a band hands its errors to the first line of the next through a ring in
// shared memory, read at least one barrier after it was written.
//
// Per warp, inputs and outputs go through two 32 x 16 staging tiles in shared
// memory (pitch 17 words: the lanes of a step hit 32 distinct banks), filled
// and drained with coalesced loads and stores once per 16 steps; the loads of
// the next 16 steps are in flight while the current ones run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "depth.h"
#include "depth_device.cuh"

namespace zg {

namespace {

constexpr int kBandLines = 32;
constexpr int kTile = kBandLines * kEdPitch;       // words per staging tile
constexpr int kTail = kEdLag * (kBandLines - 1);   // steps line 31 runs behind line 0
// Line 0 of a band reads the line above at column c + 3 on step c, written
// on step c + 3 + kTail of the previous band: spacing - kTail - 3 >= kEdChunk
// puts the write one barrier before the read.
constexpr int kMinSpacing = ((kTail + 3 + kEdChunk + kEdChunk - 1) / kEdChunk) * kEdChunk;
constexpr int kMaxWarps = 32;
constexpr size_t kMaxSmem = 227 * 1024;

// Where a warp is on the current chunk: the band it owns and the band's
// step; live while that band has work left. Warp w starts at global step
// w * spacing and moves to band + warps every `cycle` steps.
struct Where {
	int band, step;
	bool live;
};

__device__ __forceinline__ bool where_live(const Where &x, int rel, const EdPlane &p)
{
	return rel >= 0 && x.band < p.bands && x.step < kTail + p.width;
}

// The next chunk's position (rel: global step - w * spacing, advanced here).
__device__ __forceinline__ void where_next(Where &x, int &rel, int w, int nw, const EdPlane &p)
{
	rel += kEdChunk;
	if (rel == 0) {
		x.band = w;
		x.step = 0;
	} else if (rel > 0) {
		x.step += kEdChunk;
		if (x.step >= p.cycle) {
			x.step -= p.cycle;
			x.band += nw;
		}
	}
	x.live = where_live(x, rel, p);
}

template <class T, class U>
__global__ void __launch_bounds__(kMaxWarps * 32) ed_kernel(const __grid_constant__ EdLaunch L)
{
	extern __shared__ __align__(16) float ed_smem[];
	const EdPlane &p = L.planes[blockIdx.x];
	const int nw = L.warps, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int per_warp = 2 * kTile + L.ring;
	float *tile_in = ed_smem + w * per_warp;
	uint32_t *tile_out = reinterpret_cast<uint32_t *>(tile_in + kTile);
	float *ring = tile_in + 2 * kTile;
	const float *ring_above = ed_smem + ((w + nw - 1) % nw) * per_warp + 2 * kTile;
	const int rmask = L.ring - 1;
	const int W = p.width, H = p.height;
	const float scale = p.scale, offset = p.offset, vmax = p.vmax;
	// staging: transfer j of a lane covers line 2j + half of the band, step t16
	const int half = lane >> 4, t16 = lane & 15;

	T pre[kEdChunk];
	auto fetch = [&](const Where &wh) {
		if (!wh.live) {
#pragma unroll
			for (int j = 0; j < kEdChunk; ++j)
				pre[j] = T{};
			return;
		}
		const int rows_left = H - wh.band * kBandLines - half;  // line 2j + half exists iff 2j < rows_left
		const char *base = static_cast<const char *>(p.src) +
		                   static_cast<ptrdiff_t>(wh.band * kBandLines + half) * p.src_stride;
		const ptrdiff_t step2 = 2 * p.src_stride;
		const int cb = wh.step + t16 - kEdLag * half;
#pragma unroll
		for (int j = 0; j < kEdChunk; ++j) {
			const int c = cb - 2 * kEdLag * j;
			const bool ok = 2 * j < rows_left && static_cast<unsigned>(c) < static_cast<unsigned>(W);
			pre[j] = ok ? reinterpret_cast<const T *>(base + j * step2)[c] : T{};
		}
	};

	// errors: left neighbour; h2 / h3 / h4 the line above at columns c + 1,
	// c, c - 1 for this step, h1 the one for the next step
	float left = 0.0f, h1 = 0.0f, h2 = 0.0f, h3 = 0.0f, h4 = 0.0f;
	int rel = -w * p.spacing;
	Where cur{ w, 0, false };
	cur.live = where_live(cur, rel, p);
	fetch(cur);
	for (int s0 = 0; s0 < p.steps; s0 += kEdChunk) {
		Where nxt = cur;
		int rel_next = rel;
		where_next(nxt, rel_next, w, nw, p);
		if (cur.live) {
			// x = sample * scale + offset, two roundings (dither.cpp:76)
#pragma unroll
			for (int j = 0; j < kEdChunk; ++j)
				tile_in[(2 * j + half) * kEdPitch + t16] =
					__fadd_rn(__fmul_rn(sample_to_float(pre[j]), scale), offset);
		}
		fetch(nxt);
		__syncwarp();
		if (cur.live) {
			if (cur.step == 0) {
				// a band starts: line 0 takes the first three errors of the
				// line above from the previous band's ring (zero above line 0)
				left = h1 = h2 = h3 = h4 = 0.0f;
				if (lane == 0 && cur.band > 0) {
					h3 = ring_above[0];
					h2 = W > 1 ? ring_above[1] : 0.0f;
					h1 = W > 2 ? ring_above[2] : 0.0f;
				}
			}
			const bool row_ok = cur.band * kBandLines + lane < H;
			const bool above = cur.band > 0;
			const int c0 = cur.step - kEdLag * lane;
			// Branch-free steps: every lane computes, inactive lanes (before
			// or after their line, or below the plane) keep a zero error.
#pragma unroll
			for (int t = 0; t < kEdChunk; ++t) {
				const int c = c0 + t;
				const bool act = row_ok && static_cast<unsigned>(c) < static_cast<unsigned>(W);
				// left * 7/16 + top-right * 3/16 + top * 5/16 + top-left *
				// 1/16, in that order (dither.cpp:78-83). zimg's sum starts
				// from 0, which only turns a -0 into +0: the sample's base is
				// never -0 (x * scale + offset with offset never -0), so a
				// zero's sign cannot reach x and the start is left out.
				float err = __fmul_rn(left, 0.4375f);
				err = __fadd_rn(err, __fmul_rn(h2, 0.1875f));
				err = __fadd_rn(err, __fmul_rn(h3, 0.3125f));
				err = __fadd_rn(err, __fmul_rn(h4, 0.0625f));
				const float x = __fadd_rn(tile_in[lane * kEdPitch + t], err);
				// std::clamp to [0, vmax] (x is never -0); a NaN clamps to 0
				// here, stores 0 as zimg's lrint does, and keeps its NaN as
				// the error below
				const float xc = fminf(fmaxf(x, 0.0f), vmax);
				// nearest even: xc + 1.5 * 2^23 has an ulp of 1 for
				// 0 <= xc < 2^22
				const float r = __fadd_rn(xc, 12582912.0f);
				const float y = __fsub_rn(r, 12582912.0f);
				tile_out[lane * kEdPitch + t] = __float_as_uint(r) & 0xFFFFu;
				const float e = act ? (x != x ? x : __fsub_rn(xc, y)) : 0.0f;
				if (lane == kBandLines - 1 && act)
					ring[c & rmask] = e;
				left = e;
				const float down = __shfl_up_sync(0xffffffffu, e, 1);
				// line 0 reads the previous band's last line instead; every
				// lane loads its slot (lanes are 3 columns apart: distinct
				// banks) and line 0 keeps it
				const int c3 = c + kEdLag;
				const float ra = ring_above[c3 & rmask];
				const float u = lane != 0 ? down : ((above && static_cast<unsigned>(c3) < static_cast<unsigned>(W)) ? ra : 0.0f);
				h4 = h3;
				h3 = h2;
				h2 = h1;
				h1 = u;
			}
		}
		__syncwarp();
		if (cur.live) {
			const int rows_left = H - cur.band * kBandLines - half;
			char *base = static_cast<char *>(p.dst) + static_cast<ptrdiff_t>(cur.band * kBandLines + half) * p.dst_stride;
			const ptrdiff_t step2 = 2 * p.dst_stride;
			const int cb = cur.step + t16 - kEdLag * half;
#pragma unroll
			for (int j = 0; j < kEdChunk; ++j) {
				const int c = cb - 2 * kEdLag * j;
				if (2 * j < rows_left && static_cast<unsigned>(c) < static_cast<unsigned>(W))
					reinterpret_cast<U *>(base + j * step2)[c] = static_cast<U>(tile_out[(2 * j + half) * kEdPitch + t16]);
			}
		}
		// ring writes of this chunk become visible to the next band's warp
		__syncthreads();
		cur = nxt;
		rel = rel_next;
	}
}

template <class T, class U>
cudaError_t launch_tu(const EdLaunch &L, size_t smem, cudaStream_t st)
{
	static bool raised = false;
	if (!raised) {
		cudaError_t e = cudaFuncSetAttribute(ed_kernel<T, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                                     static_cast<int>(kMaxSmem));
		if (e != cudaSuccess)
			return e;
		raised = true;
	}
	ed_kernel<T, U><<<L.num_planes, L.warps * 32, smem, st>>>(L);
	return cudaGetLastError();
}

template <class T>
cudaError_t launch_t(const EdLaunch &L, size_t smem, cudaStream_t st)
{
	switch (L.out_type) {
	case 0: return launch_tu<T, uint8_t>(L, smem, st);
	case 1: return launch_tu<T, uint16_t>(L, smem, st);
	default: return cudaErrorInvalidValue;
	}
}

int round_up(int v, int m)
{
	return (v + m - 1) / m * m;
}

} // namespace

size_t ed_smem_bytes(int warps, int ring)
{
	return static_cast<size_t>(warps) * (2 * kTile + ring) * sizeof(float);
}

bool ed_shape(EdPlane &p, int warps, int *ring)
{
	if (p.width <= 0 || p.height <= 0 || warps < 1 || warps > kMaxWarps)
		return false;
	p.bands = (p.height + kBandLines - 1) / kBandLines;
	long long spacing = kMinSpacing, cycle = 1LL << 30;
	int r = 32;
	if (p.bands > warps) {
		if (warps < 2)
			return false;
		// a warp's next band starts after its current one ends, and after
		// the next band's line 0 has read the whole ring
		const long long w = p.width;
		spacing = std::max<long long>(spacing, (w + kTail + 1 + warps - 1) / warps);
		spacing = std::max<long long>(spacing, (w + kEdChunk + warps - 2) / (warps - 1));
		spacing = (spacing + kEdChunk - 1) / kEdChunk * kEdChunk;
		cycle = spacing * warps;
		// the ring holds a column until line 0 of the next band has read it
		// one barrier later
		while (r < spacing - (kTail + 3) + kEdChunk && r < (1 << 20))
			r <<= 1;
	}
	if (spacing > (1 << 24) || cycle > (1LL << 30))
		return false;
	const long long steps = (static_cast<long long>(p.bands) - 1) * spacing + kTail + p.width;
	if (steps > (1LL << 30))
		return false;
	p.spacing = static_cast<int>(spacing);
	p.cycle = static_cast<int>(cycle);
	p.steps = round_up(static_cast<int>(steps), kEdChunk);
	*ring = r;
	return ed_smem_bytes(warps, r) <= kMaxSmem;
}

int ed_choose_warps(int width, int height)
{
	const int bands = (height + kBandLines - 1) / kBandLines;
	if (bands <= 1)
		return 1;
	// one step of a warp: ~190 cycles of latency, plus ~54 issued
	// instructions per warp in flight over four schedulers (fitted to
	// measured 540p, 1080p and 2160p planes at 4 to 32 warps)
	constexpr double kChain = 190.0, kIssue = 54.0;
	int best = 0;
	double best_cost = 0.0;
	for (int nw = 2; nw <= kMaxWarps; ++nw) {
		EdPlane p{};
		p.width = width;
		p.height = height;
		int ring = 0;
		if (!ed_shape(p, nw, &ring))
			continue;
		const int in_flight = std::min({ nw, bands, (kTail + width + p.spacing - 1) / p.spacing });
		const double cost = static_cast<double>(p.steps) * (kChain + in_flight * kIssue / 4.0);
		if (!best || cost < best_cost) {
			best = nw;
			best_cost = cost;
		}
	}
	return best;
}

cudaError_t launch_error_diffusion(const EdLaunch &L, cudaStream_t stream)
{
	if (L.num_planes <= 0)
		return cudaSuccess;
	if (L.num_planes > kEdMaxPlanes || L.warps < 1 || L.warps > kMaxWarps || L.ring < 1 || (L.ring & (L.ring - 1)))
		return cudaErrorInvalidValue;
	const size_t smem = ed_smem_bytes(L.warps, L.ring);
	if (smem > kMaxSmem)
		return cudaErrorInvalidValue;
	switch (L.in_type) {
	case 0: return launch_t<uint8_t>(L, smem, stream);
	case 1: return launch_t<uint16_t>(L, smem, stream);
	case 2: return launch_t<Half>(L, smem, stream);
	case 3: return launch_t<float>(L, smem, stream);
	default: return cudaErrorInvalidValue;
	}
}

} // namespace zg
