// Tensor-core u16 kernel with the two passes chained in registers (exact).
//
// Arithmetic is that of mma_kernel.cuh (re-centred fp16 samples, int16 taps
// split into two fp16 halves, fp32 accumulators that the planner proved hold
// exact integers, zimg's rounding and clamping per pass,
// resize_impl.cpp:31-42). The data flow differs: each warp owns one or two
// 16-column tiles of the CTA's strip of output columns and, per group of 16
// output rows, computes both passes itself without shared memory in between:
//
//   H first:  Dh[16 out cols][8 lines]  = Ah[16 out cols][16 in cols] * src[in cols][lines]
//             Dv[16 out rows][8 cols]   = Av[16 out rows][16 lines]   * Dh^T
//   V first:  Dv[16 out rows][8 in cols] = Av * src[lines][in cols]
//             Dh[16 out cols][8 rows]    = Ah * Dv^T
//
// The mma.m16n8k16 accumulator layout (row gid, columns 2tig, 2tig+1) is the
// layout of the B operand of the next product (k = 2tig, 2tig+1, n = gid), so
// the first product's rounded results, converted to centred fp16 pairs, are
// the second product's B fragments as they stand. Source lines stream
// through one ring of raw u16 lines per CTA (cp.async, prefetched `depth`
// groups ahead, one CTA barrier per group) and are centred to fp16 as they
// are read; results leave through per-warp staging tiles (stmatrix) as
// 16-byte rows.
#pragma once

#include "mma_kernel.cuh"

namespace zg {
namespace chain_detail {

using mma_detail::cp_async16;
using mma_detail::cp_async_commit;
using mma_detail::cp_async_wait;
using mma_detail::find_job;
using mma_detail::ldsm_x4_trans;
using mma_detail::mma16816;
using mma_detail::pack_u16x2;
using mma_detail::u16x2_to_centred_h2;
using mma_detail::wrap;

// CTA shape: 7 computing warps, two CTAs per SM. The strip of a CTA (7 warps'
// tiles) is also the strip of the warp-specialised TMA form
// (chain_tma_kernel.cuh), whose CTAs add one producer warp: 8 warps at up to
// 128 registers each, two CTAs per SM.
__host__ __device__ constexpr int warps_per_cta(bool /*h_first*/)
{
	return 7;
}
constexpr int kMaxWarps = 7;
constexpr int kTileW = 16;                 // output columns of one tile (one m16 block)

// Tiles per warp: several share the loop, the loads and the barriers, as far
// as their tap fragments fit in registers next to everything else: four for
// 16-line, 16-column windows (the 2x upscales), two for other small windows.
__host__ __device__ constexpr int tiles_per_warp(int kv, int kh)
{
	return (kv == 1 && kh == 1) ? 4 : ((kv + kh <= 3 || kh == 1) ? 2 : 1);
}
constexpr int kStageBytes = 48;            // staged row: 16 u16 + pad (stmatrix rows without bank conflicts)
constexpr int kMaxTilesPerWarp = 4;
constexpr int kTileStage = 16 * kStageBytes + 32;       // a warp's staged tiles lie 32 mod 128 bytes apart
constexpr int kWarpStage = kMaxTilesPerWarp * kTileStage;

__device__ __forceinline__ void stsm_x4(void *p, uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(p));
	asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};\n" ::"r"(s), "r"(r0), "r"(r1),
	             "r"(r2), "r"(r3)
	             : "memory");
}

__device__ __forceinline__ void stsm_x4_trans(void *p, uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3)
{
	const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(p));
	asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1, %2, %3, %4};\n" ::"r"(s), "r"(r0),
	             "r"(r1), "r"(r2), "r"(r3)
	             : "memory");
}

// Stage reads and global stores of a warp's staged tiles, one 16-byte chunk
// per lane and store: with four tiles a store covers 4 rows x 128 bytes (row
// lane >> 3, tile (lane >> 1) & 3, half lane & 1); with two, 8 rows x 64
// bytes (rows q and q + 4, q = lane >> 3, tile (lane >> 1) & 1); with one,
// 16 rows x 32 bytes (rows q', q' + 2, q' + 4, q' + 6 of phase q). The staged
// tiles lie 32 mod 128 bytes apart, so the 8 lanes of a phase always read 8
// different 16-byte bank groups.
__host__ __device__ constexpr int store_rows(int tiles)
{
	return tiles == 4 ? 4 : (tiles == 2 ? 8 : 16);
}
__device__ __forceinline__ int store_row(int tiles, int lane)
{
	return tiles == 4 ? (lane >> 3)
	                  : (tiles == 2 ? (lane >> 3) + 4 * ((lane >> 2) & 1)
	                                : ((lane >> 3) & 1) + 8 * (lane >> 4) + 2 * ((lane >> 1) & 3));
}
__device__ __forceinline__ int store_tile(int tiles, int lane)
{
	return tiles == 4 ? (lane >> 1) & 3 : (tiles == 2 ? (lane >> 1) & 1 : 0);
}

struct Item {
	const char *src;
	ptrdiff_t src_stride;
	char *dst;
	ptrdiff_t dst_stride;
	int src_w, src_h, dst_w, dst_h, vec_ok;
	int strip, c0, xlo;
	int g_begin, g_end, depth;
	// this thread's part of line copies: 16-byte chunk q0 of lines l0,
	// l0 + lpp, ... (threads with l0 >= lpp copy nothing); src_col: that
	// chunk's first sample in row 0, col_bytes of it inside the plane
	int q0, l0, lpp, gx, col_bytes;
	const char *src_col;
	float magic;
	uint32_t pmax2, bias_h2;
};

// Units t .. t_end - 1 of job J that lie in the strip of unit t: a work item.
// A job's units are its (strip, 16-row group) pairs, strip-major.
__device__ __forceinline__ Item make_item(const FusedJob &J, int t, int t_end, int strip_tiles, int nthreads)
{
	Item it;
	const int local = t - J.item_begin;
	it.strip = local / J.groups;
	it.g_begin = local - it.strip * J.groups;
	it.g_end = min(J.groups, it.g_begin + (t_end - t));
	it.src = static_cast<const char *>(J.src);
	it.src_stride = J.src_stride;
	it.dst = static_cast<char *>(J.dst);
	it.dst_stride = J.dst_stride;
	it.src_w = J.src_w;
	it.src_h = J.src_h;
	it.dst_w = J.dst_w;
	it.dst_h = J.dst_h;
	it.vec_ok = J.vec_ok;
	it.c0 = it.strip * strip_tiles * kTileW;
	it.xlo = __ldg(J.win_col + 2 * it.strip);
	const int pxa = (__ldg(J.win_col + 2 * it.strip + 1) - it.xlo + 7) & ~7;
	it.depth = J.depth;
	it.magic = J.magic;
	const uint32_t pm = static_cast<uint32_t>(J.pixel_max);
	it.pmax2 = pm | (pm << 16);
	const __half2 b = __floats2half2_rn(1024.0f + J.offset, 1024.0f + J.offset);
	it.bias_h2 = *reinterpret_cast<const uint32_t *>(&b);
	const int chunks = pxa / 8;
	it.q0 = threadIdx.x % chunks;
	it.l0 = threadIdx.x / chunks;
	it.lpp = nthreads / chunks;
	it.gx = it.xlo + it.q0 * 8;
	const int n = max(0, min(8, it.src_w - it.gx));
	it.col_bytes = n * 2;
	it.src_col = n ? it.src + static_cast<ptrdiff_t>(it.gx) * 2 : it.src;
	return it;
}

// Source lines [a, b) of the strip (raw u16, zeros outside the plane) into
// ring slots; line a goes to slot sa. b - a is less than the ring size R.
__device__ __forceinline__ void load_lines(const Item &it, int a, int b, char *ring, int R, int sa, int pitch_bytes)
{
	int y = a + it.l0;
	if (it.l0 >= it.lpp || y >= b)
		return;
	int slot = wrap(sa + it.l0, R);
	if (it.vec_ok) {
		const char *src = it.src_col + static_cast<ptrdiff_t>(y) * it.src_stride;
		const ptrdiff_t step = static_cast<ptrdiff_t>(it.lpp) * it.src_stride;
		for (; y < b; y += it.lpp, src += step) {
			const bool ok = y < it.src_h;
			cp_async16(ring + slot * pitch_bytes + it.q0 * 16, ok ? src : it.src, ok ? it.col_bytes : 0);
			slot = wrap(slot + it.lpp, R);
		}
	} else {
		for (; y < b; y += it.lpp) {
			const bool row_ok = y < it.src_h;
			const uint16_t *row = reinterpret_cast<const uint16_t *>(it.src + static_cast<ptrdiff_t>(row_ok ? y : 0) * it.src_stride);
			uint16_t *d = reinterpret_cast<uint16_t *>(ring + slot * pitch_bytes + it.q0 * 16);
#pragma unroll
			for (int e = 0; e < 8; ++e)
				d[e] = (row_ok && it.gx + e < it.src_w) ? __ldg(row + it.gx + e) : static_cast<uint16_t>(0);
			slot = wrap(slot + it.lpp, R);
		}
	}
}

__device__ __forceinline__ uint32_t centre(uint32_t q, uint32_t bias_h2)
{
	return u16x2_to_centred_h2(q, bias_h2);
}

// Vertical tap fragments of group g into a shared slot.
template <int KV>
__device__ __forceinline__ void load_vfrag(const FusedJob &J, int g, char *slot)
{
	const char *src = reinterpret_cast<const char *>(J.v_dense) + static_cast<size_t>(g) * KV * 2 * 32 * 16;
	for (int i = threadIdx.x; i < KV * 2 * 32; i += blockDim.x)
		cp_async16(slot + i * 16, src + i * 16, 16);
}

__device__ __forceinline__ void wait_groups(int pending)
{
	// cp.async.wait_group takes an immediate
	switch (pending) {
	case 0: cp_async_wait<0>(); break;
	case 1: cp_async_wait<1>(); break;
	case 2: cp_async_wait<2>(); break;
	case 3: cp_async_wait<3>(); break;
	case 4: cp_async_wait<4>(); break;
	case 5: cp_async_wait<5>(); break;
	case 6: cp_async_wait<6>(); break;
	case 7: cp_async_wait<7>(); break;
	default: cp_async_wait<8>(); break;
	}
}

// Accumulator of one 16x8 product: the hi and lo tap halves accumulate into
// the same exact-integer fp32 registers. (Separate registers per half, two
// independent mma chains, measured no faster.)
struct Acc {
	float h[4];
	__device__ __forceinline__ void init()
	{
#pragma unroll
		for (int i = 0; i < 4; ++i)
			h[i] = 8192.0f;
	}
	__device__ __forceinline__ void mma(const uint4 &hi, const uint4 &lo, uint32_t b0, uint32_t b1)
	{
		const uint32_t ah[4] = { hi.x, hi.y, hi.z, hi.w };
		const uint32_t al[4] = { lo.x, lo.y, lo.z, lo.w };
		mma16816(h, ah, b0, b1);
		mma16816(h, al, b0, b1);
	}
	__device__ __forceinline__ float operator[](int i) const { return h[i]; }
};

// Two accumulator values -> packed, clamped samples (low / high half).
__device__ __forceinline__ uint32_t pack(const Acc &a, int i, const Item &it)
{
	return pack_u16x2(a[i], a[i + 1], it.magic, it.pmax2);
}

// Two accumulator values -> the next product's centred fp16 pair.
__device__ __forceinline__ uint32_t pack_centre(const Acc &a, int i, const Item &it)
{
	return centre(pack(a, i, it), it.bias_h2);
}

// One 16-column tile of one 16-row group: both passes, then the staged
// result to the destination. ah: the tile's horizontal tap fragments, rel: its
// window start in the strip's lines, av: the group's vertical fragments.
// H first, one 16-line window per group: the H results of lines 8-15 (V
// operands of output columns 0-7 and 8-15) carried to the next group when it
// starts 8 lines later.
struct Carry {
	uint32_t b[2];
};

// Both passes of one 16-column tile of one 16-row group; m: the four packed
// 8x8 blocks of the result (row-major for H first, transposed for V first).
template <bool H_FIRST, int KV, int KH>
__device__ __forceinline__ void tile_compute(const Item &it, const char *ring, int IR, int P, int slot, int rel,
                                             const uint4 (&ah)[KH][2], const uint4 (&av)[KV][2], Carry &carry,
                                             bool reuse, uint32_t (&m)[4])
{
	const int lane = threadIdx.x & 31;
	const int gid = lane >> 2, tig = lane & 3;
	if (H_FIRST) {
		// H over the group's KV*16 lines: B = src[line gid (+8)][in cols 2tig (+8)]
		uint32_t bv[KV][2][2];
#pragma unroll
		for (int kv = 0; kv < KV; ++kv) {
			Acc dh0, dh1;  // lines 0-7, 8-15
			const bool top = !(KV == 1 && reuse);
			if (top)
				dh0.init();
			dh1.init();
			const char *r0 = ring + wrap(slot + 16 * kv + gid, IR) * P + (rel + 2 * tig) * 2;
			const char *r1 = ring + wrap(slot + 16 * kv + gid + 8, IR) * P + (rel + 2 * tig) * 2;
#pragma unroll
			for (int ks = 0; ks < KH; ++ks) {
				if (top) {
					const uint32_t b0 = centre(*reinterpret_cast<const uint32_t *>(r0 + ks * 32), it.bias_h2);
					const uint32_t b1 = centre(*reinterpret_cast<const uint32_t *>(r0 + ks * 32 + 16), it.bias_h2);
					dh0.mma(ah[ks][0], ah[ks][1], b0, b1);
				}
				const uint32_t b2 = centre(*reinterpret_cast<const uint32_t *>(r1 + ks * 32), it.bias_h2);
				const uint32_t b3 = centre(*reinterpret_cast<const uint32_t *>(r1 + ks * 32 + 16), it.bias_h2);
				dh1.mma(ah[ks][0], ah[ks][1], b2, b3);
			}
			// Dh (out col gid / gid+8, lines 2tig..) -> V operands (k = lines, n = out col)
			if (top) {
				bv[kv][0][0] = pack_centre(dh0, 0, it);
				bv[kv][1][0] = pack_centre(dh0, 2, it);
			} else {
				bv[kv][0][0] = carry.b[0];
				bv[kv][1][0] = carry.b[1];
			}
			bv[kv][0][1] = pack_centre(dh1, 0, it);
			bv[kv][1][1] = pack_centre(dh1, 2, it);
		}
		if (KV == 1) {
			carry.b[0] = bv[0][0][1];
			carry.b[1] = bv[0][1][1];
		}
		Acc dv0, dv1;  // out cols 0-7, 8-15
		dv0.init();
		dv1.init();
#pragma unroll
		for (int kv = 0; kv < KV; ++kv) {
			dv0.mma(av[kv][0], av[kv][1], bv[kv][0][0], bv[kv][0][1]);
			dv1.mma(av[kv][0], av[kv][1], bv[kv][1][0], bv[kv][1][1]);
		}
		// (out row gid / gid+8, out cols 2tig..): row-major 8x8 blocks
		m[0] = pack(dv0, 0, it);
		m[1] = pack(dv1, 0, it);
		m[2] = pack(dv0, 2, it);
		m[3] = pack(dv1, 2, it);
	} else {
		Acc dh0, dh1;  // out rows 0-7, 8-15
		dh0.init();
		dh1.init();
		// ldmatrix.trans rows: line (lane & 7) + ((lane >> 3) & 1) * 8, column + (lane >> 4) * 8
		const int krow = (lane & 7) + ((lane >> 3) & 1) * 8;
		const int coff = (rel + (lane >> 4) * 8) * 2;
#pragma unroll
		for (int ks = 0; ks < KH; ++ks) {
			Acc dv0, dv1;  // in cols 0-7, 8-15 of this k-step
			dv0.init();
			dv1.init();
#pragma unroll
			for (int kv = 0; kv < KV; ++kv) {
				uint32_t b0, b1, b2, b3;
				ldsm_x4_trans(b0, b1, b2, b3, ring + wrap(slot + 16 * kv + krow, IR) * P + coff + ks * 32);
				b0 = centre(b0, it.bias_h2);
				b1 = centre(b1, it.bias_h2);
				b2 = centre(b2, it.bias_h2);
				b3 = centre(b3, it.bias_h2);
				dv0.mma(av[kv][0], av[kv][1], b0, b1);
				dv1.mma(av[kv][0], av[kv][1], b2, b3);
			}
			// Dv (out row gid / gid+8, in cols 2tig..) -> H operands (k = in cols, n = out row)
			const uint32_t h00 = pack_centre(dv0, 0, it);
			const uint32_t h01 = pack_centre(dv1, 0, it);
			const uint32_t h10 = pack_centre(dv0, 2, it);
			const uint32_t h11 = pack_centre(dv1, 2, it);
			dh0.mma(ah[ks][0], ah[ks][1], h00, h01);
			dh1.mma(ah[ks][0], ah[ks][1], h10, h11);
		}
		// (out col gid / gid+8, out rows 2tig..): transposed 8x8 blocks
		m[0] = pack(dh0, 0, it);
		m[1] = pack(dh0, 2, it);
		m[2] = pack(dh1, 0, it);
		m[3] = pack(dh1, 2, it);
	}
}

// One lane's staged 8-sample chunk -> destination row `row`, columns col..,
// clipped to the plane.
__device__ __forceinline__ void store_chunk(const Item &it, const char *ld_addr, int row, int col)
{
	if (row < it.dst_h && col < it.dst_w) {
		const uint4 v = *reinterpret_cast<const uint4 *>(ld_addr);
		uint16_t *d = reinterpret_cast<uint16_t *>(it.dst + static_cast<ptrdiff_t>(row) * it.dst_stride) + col;
		if (it.vec_ok && col + 8 <= it.dst_w) {
			*reinterpret_cast<uint4 *>(d) = v;
		} else {
			const uint32_t w[4] = { v.x, v.y, v.z, v.w };
			for (int e = 0; e < 8 && col + e < it.dst_w; ++e)
				d[e] = static_cast<uint16_t>(w[e >> 1] >> (16 * (e & 1)));
		}
	}
}

// Kernel. Shared memory (SmemLayout): ring of raw source lines (in_off,
// in_rows x pitch), depth + 2 slots of vertical tap fragments (vcoef_off),
// one 16-row staging tile per warp (tile_off), the segment's group bases
// (vbase_off). A warp may still compute group k while others issue the loads
// of group k + 1 + depth: the planner sizes the ring and the slots for that.
template <bool H_FIRST, int KV, int KH>
__global__ void __launch_bounds__(warps_per_cta(H_FIRST) * 32, 2)
chain_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_items, const __grid_constant__ FusedJob single,
             const __grid_constant__ SmemLayout L)
{
	extern __shared__ float4 smem4[];
	char *smem = reinterpret_cast<char *>(smem4);
	char *ring = smem + L.in_off;
	char *vslots = smem + L.vcoef_off;
	int *vb = reinterpret_cast<int *>(smem + L.vbase_off);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	char *stage = smem + L.tile_off + warp * tiles_per_warp(KV, KH) * kTileStage;
	const int IR = L.in_rows;
	const int P = L.pitch * 2;
	constexpr int kSlotBytes = KV * 2 * 32 * 16;
	constexpr int kTilesPerWarp = tiles_per_warp(KV, KH);
	constexpr int kWarps = warps_per_cta(H_FIRST);
	constexpr int kThreads = kWarps * 32;
	constexpr int kStripTiles = kWarps * kTilesPerWarp;
	// stmatrix address of this lane
	char *st_addr = stage + (((lane >> 4) << 3) + (lane & 7)) * kStageBytes + ((lane >> 3) & 1) * 16;
	// Stage reads and global stores, one 16-byte chunk per lane (store_map).
	constexpr int kStoreRows = store_rows(kTilesPerWarp);
	constexpr int kStores = 16 / kStoreRows;
	const int st_row = store_row(kTilesPerWarp, lane);
	const int st_tile = store_tile(kTilesPerWarp, lane);
	const char *ld_addr = stage + st_tile * kTileStage + st_row * kStageBytes + (lane & 1) * 16;

	const int S = L.depth + 2;  // fragment slots in rotation

	// lines never written by a load still hold finite values
	for (int i = threadIdx.x; i < L.in_rows * P / 16; i += kThreads)
		reinterpret_cast<float4 *>(ring)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
	__syncthreads();

	// this CTA's equal share of the launch's units, in job / strip / group
	// order: whole strips where they fit, split at most at its two ends
	const int t_end = static_cast<int>(static_cast<long long>(blockIdx.x + 1) * total_items / gridDim.x);
	for (int t = static_cast<int>(static_cast<long long>(blockIdx.x) * total_items / gridDim.x); t < t_end;) {
		const FusedJob *Jp = jobs ? &jobs[find_job(jobs, num_jobs, t)] : &single;
		const Item it = make_item(*Jp, t, t_end, kStripTiles, kThreads);
		t += it.g_end - it.g_begin;
		for (int g = it.g_begin + threadIdx.x; g < it.g_end; g += kThreads)
			vb[g - it.g_begin] = __ldg(Jp->v_base + g);

		// this warp's tiles of 16 output columns: horizontal tap fragments and window starts
		const int ntiles = (it.dst_w + kTileW - 1) / kTileW;
		const int tile0 = it.strip * kStripTiles + warp * kTilesPerWarp;
		uint4 ah[kTilesPerWarp][KH][2];
		int rel[kTilesPerWarp];
		Carry carry[kTilesPerWarp];
		// this lane's destination chunk in the item's first group, advanced by
		// 16 rows per group; plain 16-byte stores where it is inside the plane
		const int st_col = (tile0 + st_tile) * kTileW + (lane & 1) * 8;
		const bool wide = it.vec_ok && st_col + 8 <= it.dst_w;
		char *drow = it.dst + static_cast<ptrdiff_t>(it.g_begin * 16 + st_row) * it.dst_stride +
		             static_cast<ptrdiff_t>(st_col) * 2;
		const ptrdiff_t group_step = 16 * it.dst_stride;
		const ptrdiff_t store_step = kStoreRows * it.dst_stride;
#pragma unroll
		for (int j = 0; j < kTilesPerWarp; ++j) {
			const int tile = min(tile0 + j, ntiles - 1);
			const uint4 *hf = reinterpret_cast<const uint4 *>(Jp->h_taps) + static_cast<size_t>(tile) * KH * 2 * 32 + lane;
#pragma unroll
			for (int ks = 0; ks < KH; ++ks) {
				ah[j][ks][0] = __ldg(hf + (ks * 2 + 0) * 32);
				ah[j][ks][1] = __ldg(hf + (ks * 2 + 1) * 32);
			}
			rel[j] = __ldg(Jp->h_left + tile) - it.xlo;
		}
		__syncthreads();

		const int D = it.depth;
		const int ngroups = it.g_end - it.g_begin;
		const char *vtab = reinterpret_cast<const char *>(Jp->v_dense);
		int issued_hi = vb[0];
		int issued_slot = wrap(vb[0] % IR, IR);
		// group k: new lines up to vb[k] + 16 KV, fragments into the next of S slots
		int fetch_slot = 0, read_slot = 0;
		auto issue = [&](int k) {
			const int hi = vb[k] + 16 * KV;
			if (hi > issued_hi) {
				load_lines(it, issued_hi, hi, ring, IR, issued_slot, P);
				issued_slot = wrap(issued_slot + (hi - issued_hi), IR);
				issued_hi = hi;
			}
			char *vslot = vslots + fetch_slot * kSlotBytes;
			fetch_slot = fetch_slot + 1 == S ? 0 : fetch_slot + 1;
			const char *vsrc = vtab + static_cast<size_t>(it.g_begin + k) * kSlotBytes;
			for (int i = threadIdx.x; i < KV * 2 * 32; i += kThreads)
				cp_async16(vslot + i * 16, vsrc + i * 16, 16);
		};

		// prologue: groups 0 .. D-1 in flight, one commit group each
		for (int k = 0; k < D; ++k) {
			if (k < ngroups)
				issue(k);
			cp_async_commit();
		}

		int cur_vb = vb[0];
		int cur_slot = wrap(cur_vb % IR, IR);
		for (int k = 0; k < ngroups; ++k) {
			if (k + D < ngroups)
				issue(k + D);
			cp_async_commit();
			wait_groups(D);
			__syncthreads();

			const int vbk = vb[k];
			const bool reuse = H_FIRST && KV == 1 && k > 0 && vbk - cur_vb == 8;
			cur_slot = wrap(cur_slot + (vbk - cur_vb), IR);
			cur_vb = vbk;
			if (tile0 * kTileW < it.dst_w) {
				const uint4 *avs = reinterpret_cast<const uint4 *>(vslots + read_slot * kSlotBytes) + lane;
				uint4 av[KV][2];
#pragma unroll
				for (int kv = 0; kv < KV; ++kv) {
					av[kv][0] = avs[(kv * 2 + 0) * 32];
					av[kv][1] = avs[(kv * 2 + 1) * 32];
				}
				// the tiles' products interleave; stores follow
				uint32_t m[kTilesPerWarp][4];
#pragma unroll
				for (int j = 0; j < kTilesPerWarp; ++j)
					tile_compute<H_FIRST, KV, KH>(it, ring, IR, P, cur_slot, rel[j], ah[j], av, carry[j], reuse, m[j]);
#pragma unroll
				for (int j = 0; j < kTilesPerWarp; ++j) {
					char *sa = st_addr + j * kTileStage;
					if (H_FIRST)
						stsm_x4(sa, m[j][0], m[j][1], m[j][2], m[j][3]);
					else
						stsm_x4_trans(sa, m[j][0], m[j][1], m[j][2], m[j][3]);
				}
				__syncwarp();
				const bool rows_in = (it.g_begin + k + 1) * 16 <= it.dst_h;
				if (wide && rows_in) {
#pragma unroll
					for (int i = 0; i < kStores; ++i)
						*reinterpret_cast<uint4 *>(drow + i * store_step) =
							*reinterpret_cast<const uint4 *>(ld_addr + i * kStoreRows * kStageBytes);
				} else {
#pragma unroll
					for (int i = 0; i < kStores; ++i)
						store_chunk(it, ld_addr + i * kStoreRows * kStageBytes,
						            (it.g_begin + k) * 16 + st_row + i * kStoreRows, st_col);
				}
				__syncwarp();
			}
			read_slot = read_slot + 1 == S ? 0 : read_slot + 1;
			drow += group_step;
		}
		cp_async_wait<0>();
		__syncthreads();  // the next item rewrites the group bases and the ring
	}
}

} // namespace chain_detail
} // namespace zg
