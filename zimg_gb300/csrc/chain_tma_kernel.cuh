// Chained tensor-core u16 kernel, warp-specialised TMA form.
//
// Arithmetic is that of chain_kernel.cuh (re-centred fp16 samples, int16
// taps split into two exact fp16 halves, fp32 accumulators that the planner
// proved hold exact integers, zimg's rounding and clamping per pass,
// resize_impl.cpp:31-59,78-95), and so are the 16x16 output tiles, the tap
// fragments and the strip plan. What differs is the feeding and the control
// flow, cut to the few instructions a tile needs:
//
//  - One producer warp (one lane) brings every group's data into shared
//    memory: 16-line blocks of the strip's source columns as 2-D tensor
//    copies (cp.async.bulk.tensor) into a ring of 2^n blocks, and the group's
//    vertical tap fragments as one bulk copy into a stage. Group g of the
//    CTA's pipeline uses stage g mod NS: a "full" mbarrier whose transaction
//    count covers the group's copies, and an "empty" mbarrier on which every
//    consumer warp arrives once it has read the group.
//  - Seven consumer warps only compute and store: per group, one wait, the
//    vertical fragments, the tiles of the warp (one or two of 16 columns),
//    one arrive, the stores. Line addresses are ring offsets under a mask,
//    computed once per group for all tiles; whether a group reuses the
//    previous group's horizontal products (its window starts 8 lines lower)
//    is a warp-uniform branch between two unrolled bodies.
//  - Rounding is one paired fp32 multiply-add per two samples and one
//    s16x2 minimum with relu (pack_u16x2).
//  - Source blocks wholly below the plane are not copied: the producer
//    writes them as zero lines before it arrives on the group's barrier.
//  - Every mbarrier wait is bounded (g_chain_wait_ns, default 0.25 s). A wait
//    that runs out records its cause in g_chain_pipeline_error, the CTA
//    stops, and the producer first waits (again bounded) for the copies it
//    still has in flight. A test hook (g_chain_drop_group) makes CTA 0's
//    producer skip one group without arming its stage, so that a test can
//    see a consumer wait run out and the kernel return.
#pragma once

#include <cuda.h>

#include "chain_kernel.cuh"
#include "pipeline.cuh"
#include "work_chunks.cuh"

namespace zg {
namespace chain_detail {

constexpr int kBlockLines = 16;                     // source lines per tensor copy
constexpr int kWsWarps = warps_per_cta(true);      // consumer warps per CTA

// Nonzero after a pipeline wait ran out: 1 = a group's copies never landed,
// 2 = a buffer was never released, 3 = ring too small for one group.
__device__ int g_chain_pipeline_error;
// Wait limit in ns (0: kWaitNs) and the test hook described above (-1: off).
__device__ unsigned long long g_chain_wait_ns;
__device__ int g_chain_drop_group = -1;

__host__ __device__ constexpr int tma_threads(bool /*h_first*/)
{
	return (kWsWarps + 1) * 32;
}

__device__ __forceinline__ bool mbar_wait_for(uint64_t *bar, unsigned parity, unsigned long long limit)
{
	const unsigned a = smem_addr(bar);
	unsigned long long t0 = 0;
	for (unsigned i = 0;; ++i) {
		unsigned done;
		asm volatile("{\n"
		             "  .reg .pred p;\n"
		             "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
		             "  selp.u32 %0, 1, 0, p;\n"
		             "}\n"
		             : "=r"(done)
		             : "r"(a), "r"(parity)
		             : "memory");
		if (done)
			return true;
		if ((i & 15) == 0) {
			const unsigned long long t = global_ns();
			if (i == 0)
				t0 = t;
			else if (t - t0 > limit)
				return false;
		}
	}
}

__device__ __forceinline__ uint32_t lds32(const char *p)
{
	return *reinterpret_cast<const uint32_t *>(p);
}

// D = A * B + 8192 (all four accumulators), m16n8k16 f16 -> f32
__device__ __forceinline__ void mma_init(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1, float c)
{
	asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
	    "{%10, %10, %10, %10};\n"
	             : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
	             : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(c));
}

// Accumulate both tap halves (hi, lo) of one 16x16 fragment pair; `first`
// starts the accumulators at 8192.
__device__ __forceinline__ void mma2(float (&d)[4], const uint4 &hi, const uint4 &lo, uint32_t b0, uint32_t b1,
                                     bool first)
{
	const uint32_t ah[4] = { hi.x, hi.y, hi.z, hi.w };
	const uint32_t al[4] = { lo.x, lo.y, lo.z, lo.w };
	if (first)
		mma_init(d, ah, b0, b1, 8192.0f);
	else
		mma16816(d, ah, b0, b1);
	mma16816(d, al, b0, b1);
}

struct Epi {
	float magic;
	uint32_t pmax2, bias_h2;
	__device__ __forceinline__ uint32_t pack(const float (&a)[4], int i) const
	{
		return pack_u16x2(a[i], a[i + 1], magic, pmax2);
	}
	__device__ __forceinline__ uint32_t pack_centre(const float (&a)[4], int i) const
	{
		return u16x2_to_centred_h2(pack(a, i), bias_h2);
	}
	__device__ __forceinline__ uint32_t centre(uint32_t q) const
	{
		return u16x2_to_centred_h2(q, bias_h2);
	}
};

// H first, horizontal stage: the horizontal products of the 8-line blocks of
// the group's window (blocks i = 0 .. 2 KV - 1, lines line0 + 8 i ..) for the
// warp's T tiles, rounded and centred into the vertical pass's operands:
// blk[j][i][c] holds block i of tile j for its output columns 8c .. 8c + 7
// (k = lines 2tig, 2tig + 1, n = out col gid, as the mma accumulator leaves
// them). Blocks i < keep were taken over from the previous group and are not
// recomputed. colb[j]: tile j's byte offset of its window's input column 2tig
// in a line. Each step runs over all tiles before the next, so that the
// tiles' dependency chains overlap in issue order.
template <int KV, int KH, int T, int KEEP>
__device__ __forceinline__ void hfirst_h(const char *ring, unsigned line0, unsigned line_mask, int P, int lrow,
                                         const uint32_t (&colb)[T], const uint4 (&ah)[T][KH][2],
                                         uint32_t (&blk)[T][2 * KV][2], int keep, const Epi &e)
{
#pragma unroll
	for (int i = 0; i < 2 * KV; ++i) {
		// KEEP >= 0: the number of kept blocks known at compile time
		if (KEEP >= 0 ? i < KEEP : i < keep)
			continue;
		const char *row = ring + ((line0 + 8 * i + lrow) & line_mask) * P;
		float dh[T][4];
#pragma unroll
		for (int ks = 0; ks < KH; ++ks) {
			uint32_t b[T][2];
#pragma unroll
			for (int j = 0; j < T; ++j) {
				b[j][0] = lds32(row + colb[j] + ks * 32);
				b[j][1] = lds32(row + colb[j] + ks * 32 + 16);
			}
#pragma unroll
			for (int j = 0; j < T; ++j)
				mma2(dh[j], ah[j][ks][0], ah[j][ks][1], e.centre(b[j][0]), e.centre(b[j][1]), ks == 0);
		}
#pragma unroll
		for (int j = 0; j < T; ++j) {
			blk[j][i][0] = e.pack_centre(dh[j], 0);
			blk[j][i][1] = e.pack_centre(dh[j], 2);
		}
	}
}

// Window moved by d 8-line blocks: block i becomes block i - d.
template <int KV, int T>
__device__ __forceinline__ void shift_blocks(uint32_t (&blk)[T][2 * KV][2], int d)
{
	for (int s = 0; s < d; ++s) {
#pragma unroll
		for (int j = 0; j < T; ++j)
#pragma unroll
			for (int i = 0; i + 1 < 2 * KV; ++i) {
				blk[j][i][0] = blk[j][i + 1][0];
				blk[j][i][1] = blk[j][i + 1][1];
			}
	}
}

// H first, vertical stage: the vertical products of the warp's tiles, two
// tiles at a time, each pair rounded and staged (row-major 8x8 blocks: out
// row gid / gid+8, out cols 2tig..) before the next.
template <int KV, int T>
__device__ __forceinline__ void hfirst_v(const uint32_t (&blk)[T][2 * KV][2], const uint4 (&av)[KV][2], char *st_addr,
                                         const Epi &e)
{
	constexpr int P = T < 2 ? T : 2;
#pragma unroll
	for (int j0 = 0; j0 < T; j0 += P) {
		float dv0[P][4], dv1[P][4];  // out cols 0-7, 8-15
#pragma unroll
		for (int kv = 0; kv < KV; ++kv) {
#pragma unroll
			for (int q = 0; q < P; ++q) {
				mma2(dv0[q], av[kv][0], av[kv][1], blk[j0 + q][2 * kv][0], blk[j0 + q][2 * kv + 1][0], kv == 0);
				mma2(dv1[q], av[kv][0], av[kv][1], blk[j0 + q][2 * kv][1], blk[j0 + q][2 * kv + 1][1], kv == 0);
			}
		}
#pragma unroll
		for (int q = 0; q < P; ++q)
			stsm_x4(st_addr + (j0 + q) * kTileStage, e.pack(dv0[q], 0), e.pack(dv1[q], 0), e.pack(dv0[q], 2),
			        e.pack(dv1[q], 2));
	}
}

// V first: the warp's T tiles of one group, staged as they finish. roff[kv]:
// byte offset in the ring of this lane's ldmatrix row (line (lane & 7) +
// ((lane >> 3) & 1) * 8 of window block kv); colb[j]: tile j's byte offset of
// its column (lane >> 4) * 8.
template <int KV, int KH, int T>
__device__ __forceinline__ void vfirst_tiles(const char *ring, const uint32_t (&roff)[KV], const uint32_t (&colb)[T],
                                             const uint4 (&ah)[T][KH][2], const uint4 (&av)[KV][2], char *st_addr,
                                             const Epi &e)
{
	float dh0[T][4], dh1[T][4];  // out rows 0-7, 8-15
#pragma unroll
	for (int ks = 0; ks < KH; ++ks) {
		float dv0[T][4], dv1[T][4];  // in cols 0-7, 8-15 of this k-step
#pragma unroll
		for (int kv = 0; kv < KV; ++kv) {
			uint32_t b[T][4];
#pragma unroll
			for (int j = 0; j < T; ++j)
				mma_detail::ldsm_x4_trans(b[j][0], b[j][1], b[j][2], b[j][3], ring + roff[kv] + colb[j] + ks * 32);
#pragma unroll
			for (int j = 0; j < T; ++j) {
				mma2(dv0[j], av[kv][0], av[kv][1], e.centre(b[j][0]), e.centre(b[j][1]), kv == 0);
				mma2(dv1[j], av[kv][0], av[kv][1], e.centre(b[j][2]), e.centre(b[j][3]), kv == 0);
			}
		}
		// Dv (out row gid / gid+8, in cols 2tig..) -> H operands (k = in cols, n = out row)
#pragma unroll
		for (int j = 0; j < T; ++j) {
			const uint32_t h00 = e.pack_centre(dv0[j], 0);
			const uint32_t h01 = e.pack_centre(dv1[j], 0);
			const uint32_t h10 = e.pack_centre(dv0[j], 2);
			const uint32_t h11 = e.pack_centre(dv1[j], 2);
			mma2(dh0[j], ah[j][ks][0], ah[j][ks][1], h00, h01, ks == 0);
			mma2(dh1[j], ah[j][ks][0], ah[j][ks][1], h10, h11, ks == 0);
		}
	}
	// (out col gid / gid+8, out rows 2tig..): transposed 8x8 blocks
#pragma unroll
	for (int j = 0; j < T; ++j)
		stsm_x4_trans(st_addr + j * kTileStage, e.pack(dh0[j], 0), e.pack(dh0[j], 2), e.pack(dh1[j], 0),
		              e.pack(dh1[j], 2));
}

// Per-CTA pipeline state, shared by the items a CTA processes. Shared memory
// (SmemLayout, from a 128-byte aligned base): ring of NB = in_rows /
// kBlockLines blocks of source lines, NB a power of two (in_off); NS =
// ring_rows stages of vertical tap fragments (vcoef_off); the staged tiles of
// each consumer warp (tile_off); the item's group bases (vbase_off); NS full
// and NS empty mbarriers (stage_off).
struct Pipe {
	char *smem, *ring, *vslots;
	int *vb;
	uint64_t *full, *empty;
	int *abort_item;
	int NS, NB, P, warp, lane;
	unsigned line_mask;
	bool producer;
	unsigned long long wait_ns;
	// groups since the kernel started: `base` is the current item's first
	// group; the producer also tracks `released` (groups every consumer warp
	// has finished, as observed on the empty barriers) and `issued`
	unsigned base, released, issued;
	int error;
};

__device__ __forceinline__ void pipe_init(Pipe &p, float4 *smem4, const SmemLayout &L, int *abort_item)
{
	// tensor copies land on 128-byte boundaries: align the layout's base (by
	// an offset from the shared array, so that every access through these
	// pointers stays a shared-memory access)
	char *smem = reinterpret_cast<char *>(smem4);
	smem += (128u - (smem_addr(smem) & 127u)) & 127u;
	p.smem = smem;
	p.ring = smem + L.in_off;
	p.vslots = smem + L.vcoef_off;
	p.vb = reinterpret_cast<int *>(smem + L.vbase_off);
	p.full = reinterpret_cast<uint64_t *>(smem + L.stage_off);
	p.NS = L.ring_rows;
	p.empty = p.full + p.NS;
	p.abort_item = abort_item;
	p.warp = threadIdx.x >> 5;
	p.lane = threadIdx.x & 31;
	p.producer = p.warp == kWsWarps;
	p.NB = L.in_rows / kBlockLines;
	p.line_mask = static_cast<unsigned>(L.in_rows - 1);
	p.P = L.pitch * 2;
	p.wait_ns = g_chain_wait_ns ? g_chain_wait_ns : kWaitNs;
	p.base = p.released = p.issued = 0;
	p.error = 0;
	if (threadIdx.x == 0) {
		for (int s = 0; s < p.NS; ++s) {
			mbar_init(&p.full[s], 1);
			mbar_init(&p.empty[s], kWsWarps);
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		*abort_item = 0;
	}
	__syncthreads();
}

// Before the CTA leaves: a wait that ran out is recorded, and the producer
// first waits (bounded) for its copies still in flight: only the last NS
// issued groups can have any (an earlier group's stage was reissued only
// after every consumer had read it); a dropped group has none.
__device__ __forceinline__ void pipe_finish(Pipe &p)
{
	if (p.producer && p.lane == 0 && (p.error || *p.abort_item)) {
		atomicCAS(&g_chain_pipeline_error, 0, p.error ? p.error : 1);
		const int drop = blockIdx.x == 0 ? g_chain_drop_group : -1;
		for (unsigned g = p.issued > static_cast<unsigned>(p.NS) ? p.issued - p.NS : 0; g < p.issued; ++g)
			if (static_cast<int>(g) != drop)
				mbar_wait_for(&p.full[g % p.NS], (g / p.NS) & 1, p.wait_ns);
	} else if (!p.producer && p.lane == 0 && p.error) {
		atomicCAS(&g_chain_pipeline_error, 0, p.error);
	}
}

// One item: groups g_begin .. g_begin + ngroups - 1 of strip `strip` of job
// J, the group bases already in p.vb. The producer warp brings the data in;
// the consumer warps compute and store. Both sides pass one CTA barrier
// (group bases visible, the previous item finished).
// SPECIALISE: compile-time bodies for the common reuse cases (the
// single-variant kernels; the mixed kernel keeps one body per variant).
template <bool H_FIRST, int KV, int KH, bool SPECIALISE>
__device__ __forceinline__ void chain_item(Pipe &p, const SmemLayout &L, const FusedJob &J, const void *tmap, int strip,
                                           int g_begin, int ngroups)
{
	constexpr int kSlotBytes = KV * 2 * 32 * 16;
	constexpr int T = tiles_per_warp(KV, KH);
	constexpr int kStripTiles = kWsWarps * T;
	const int NS = p.NS, NB = p.NB, P = p.P, warp = p.warp, lane = p.lane;
	const unsigned line_mask = p.line_mask;
	const unsigned long long wait_ns = p.wait_ns;
	char *const smem = p.smem;
	char *const ring = p.ring;
	char *const vslots = p.vslots;
	const int *const vb = p.vb;
	uint64_t *const full = p.full;
	uint64_t *const empty = p.empty;
	const bool producer = p.producer;
	if (producer) {
		__syncthreads();  // group bases visible; every warp is done with the previous item
		if (lane == 0 && !p.error) {
						const char *vtab = reinterpret_cast<const char *>(J.v_dense);
			const int xlo = __ldg(J.win_col + 2 * strip);
			const int drop = blockIdx.x == 0 ? g_chain_drop_group : -1;
			// next source block to load; first group of the item whose
			// window starts at or after the block being replaced
			int next_blk = vb[0] / kBlockLines;
			int gneed = 0;
			// advance `p.released` to n; false when a wait ran out
			int rel_s = static_cast<int>(p.released % NS);
			unsigned rel_ph = (p.released / NS) & 1;
			auto release_to = [&](unsigned n) -> bool {
				while (p.released < n) {
					if (!mbar_wait_for(&empty[rel_s], rel_ph, wait_ns))
						return false;
					++p.released;
					if (++rel_s == NS) {
						rel_s = 0;
						rel_ph ^= 1;
					}
				}
				return true;
			};
			int s = static_cast<int>(p.base % NS);
			const int in_blks = (J.src_h + kBlockLines - 1) / kBlockLines;
			asm volatile("prefetch.tensormap [%0];\n" ::"l"(tmap) : "memory");
			for (int k = 0; k < ngroups; ++k, s = s + 1 == NS ? 0 : s + 1) {
				const unsigned g = p.base + k;
				// the stage's fragment slot was last read by group g - NS
				if (g >= static_cast<unsigned>(NS) && !release_to(g - NS + 1)) {
					p.error = 2;
					break;
				}
				const int last_blk = (vb[k] + 16 * KV - 1) / kBlockLines;
				for (int b = next_blk; b <= last_blk && !p.error; ++b) {
					// ring block b mod NB held block b - NB, which groups
					// read up to the first one whose window starts past it
					while (gneed < ngroups && vb[gneed] < (b - NB + 1) * kBlockLines)
						++gneed;
					if (gneed > k)
						p.error = 3;  // the ring cannot hold one window
					else if (!release_to(p.base + gneed))
						p.error = 2;
				}
				if (p.error)
					break;
				if (static_cast<int>(g) == drop) {
					// test hook: this group's stage is never armed
					p.issued = g + 1;
					continue;
				}
				// blocks wholly below the plane (windows are padded to
				// 16 KV lines; their taps there are zero) become zero
				// lines, written here, not copied
				const int copy_end = min(last_blk + 1, in_blks);
				const int ncopy = max(0, copy_end - next_blk);
				for (int b = max(next_blk, in_blks); b <= last_blk; ++b) {
					float4 *z = reinterpret_cast<float4 *>(ring + (b & (NB - 1)) * kBlockLines * P);
					for (int i = 0; i < kBlockLines * P / 16; ++i)
						z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
					// later tensor copies into this block come after these stores
					asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
				}
				mbar_arrive_expect_tx(&full[s], static_cast<unsigned>(kSlotBytes + ncopy * kBlockLines * P));
				for (int b = next_blk; b < copy_end; ++b)
					tma_load_2d(ring + (b & (NB - 1)) * kBlockLines * P, tmap, xlo, b * kBlockLines, &full[s]);
				bulk_load(vslots + s * kSlotBytes, vtab + static_cast<size_t>(g_begin + k) * kSlotBytes,
				          kSlotBytes, &full[s]);
				next_blk = max(next_blk, last_blk + 1);
				p.issued = g + 1;
			}
			if (p.error)
				*p.abort_item = 1;  // benign race: every writer stores 1
		}
	} else {
		const int xlo = __ldg(J.win_col + 2 * strip);
		const int gid = lane >> 2, tig = lane & 3;
		const int ntiles = (J.dst_w + kTileW - 1) / kTileW;
		const int tile0 = strip * kStripTiles + warp * T;
		const bool active = tile0 * kTileW < J.dst_w;
		uint4 ah[T][KH][2];
		uint32_t colb[T];
		uint32_t blk[T][2 * KV][2];  // H first: the window's 8-line blocks (hfirst_h)
#pragma unroll
		for (int j = 0; j < T; ++j) {
			const int tile = min(tile0 + j, ntiles - 1);
			const uint4 *hf = reinterpret_cast<const uint4 *>(J.h_taps) + static_cast<size_t>(tile) * KH * 2 * 32 + lane;
#pragma unroll
			for (int ks = 0; ks < KH; ++ks) {
				ah[j][ks][0] = __ldg(hf + (ks * 2 + 0) * 32);
				ah[j][ks][1] = __ldg(hf + (ks * 2 + 1) * 32);
			}
			const int rel = __ldg(J.h_left + tile) - xlo;
			colb[j] = H_FIRST ? static_cast<uint32_t>((rel + 2 * tig) * 2)
			                  : static_cast<uint32_t>((rel + (lane >> 4) * 8) * 2);
#pragma unroll
			for (int i = 0; i < 2 * KV; ++i)
				blk[j][i][0] = blk[j][i][1] = 0;
		}
		Epi e;
		e.magic = J.magic;
		const uint32_t pm = static_cast<uint32_t>(J.pixel_max);
		e.pmax2 = pm | (pm << 16);
		{
			const __half2 b = __floats2half2_rn(1024.0f + J.offset, 1024.0f + J.offset);
			e.bias_h2 = *reinterpret_cast<const uint32_t *>(&b);
		}
		// stores: one 16-byte chunk per lane and store (see chain_kernel.cuh)
		char *stage = smem + L.tile_off + warp * T * kTileStage;
		char *st_addr = stage + (((lane >> 4) << 3) + (lane & 7)) * kStageBytes + ((lane >> 3) & 1) * 16;
		constexpr int kStoreRows = store_rows(T);
		constexpr int kStores = 16 / kStoreRows;
		const int st_row = store_row(T, lane);
		const int st_tile = store_tile(T, lane);
		const char *ld_addr = stage + st_tile * kTileStage + st_row * kStageBytes + (lane & 1) * 16;
		const int st_col = (tile0 + st_tile) * kTileW + (lane & 1) * 8;
		const bool wide = J.vec_ok && st_col + 8 <= J.dst_w;
		char *const dst = static_cast<char *>(J.dst);
		const ptrdiff_t dst_stride = J.dst_stride;
		char *drow = dst + static_cast<ptrdiff_t>(g_begin * 16 + st_row) * dst_stride + static_cast<ptrdiff_t>(st_col) * 2;
		const ptrdiff_t group_step = 16 * dst_stride;
		const ptrdiff_t store_step = kStoreRows * dst_stride;
		// groups whose 16 rows all lie in the plane
		const int full_groups = J.dst_h / 16 - g_begin;
		// this lane's line in each 16-line window block
		const int lrow = H_FIRST ? gid : (lane & 7) + ((lane >> 3) & 1) * 8;
		__syncthreads();  // group bases visible; every warp is done with the previous item

		int prev_vb = vb[0];
		int s = static_cast<int>(p.base % NS);
		unsigned ph = (p.base / NS) & 1;
		for (int k = 0; k < ngroups; ++k) {
			// every lane polls; the warp goes on only when all saw the copies land
			if (!__all_sync(0xffffffffu, mbar_wait_for(&full[s], ph, wait_ns))) {
				p.error = 1;
				*p.abort_item = 1;  // benign race: every writer stores 1
				break;
			}
			const int vbk = vb[k];
			if (active) {
				const uint4 *avs = reinterpret_cast<const uint4 *>(vslots + s * kSlotBytes) + lane;
				uint4 av[KV][2];
				if (H_FIRST) {
					// blocks of the previous group's window that this one keeps:
					// compile-time bodies (SPECIALISE) for a move by one block (2x
					// upscales) and for none kept
					const int moved = vbk - prev_vb;
					const unsigned line0 = static_cast<unsigned>(vbk);
					const bool slide = k > 0 && (moved & 7) == 0 && moved < 16 * KV;
					if (SPECIALISE && slide && moved == 8) {
						shift_blocks<KV, T>(blk, 1);
						hfirst_h<KV, KH, T, 2 * KV - 1>(ring, line0, line_mask, P, lrow, colb, ah, blk, 0, e);
					} else if (SPECIALISE && !slide) {
						hfirst_h<KV, KH, T, 0>(ring, line0, line_mask, P, lrow, colb, ah, blk, 0, e);
					} else {
						if (slide)
							shift_blocks<KV, T>(blk, moved >> 3);
						hfirst_h<KV, KH, T, -1>(ring, line0, line_mask, P, lrow, colb, ah, blk,
						                        slide ? 2 * KV - (moved >> 3) : 0, e);
					}
#pragma unroll
					for (int kv = 0; kv < KV; ++kv) {
						av[kv][0] = avs[(kv * 2 + 0) * 32];
						av[kv][1] = avs[(kv * 2 + 1) * 32];
					}
					// the group's shared data are in registers: release the stage
					__syncwarp();
					if (lane == 0)
						mbar_arrive(&empty[s]);
					hfirst_v<KV, T>(blk, av, st_addr, e);
				} else {
#pragma unroll
					for (int kv = 0; kv < KV; ++kv) {
						av[kv][0] = avs[(kv * 2 + 0) * 32];
						av[kv][1] = avs[(kv * 2 + 1) * 32];
					}
					uint32_t roff[KV];
#pragma unroll
					for (int kv = 0; kv < KV; ++kv)
						roff[kv] = ((static_cast<unsigned>(vbk + 16 * kv + lrow)) & line_mask) * P;
					vfirst_tiles<KV, KH, T>(ring, roff, colb, ah, av, st_addr, e);
					// the group's shared data are in registers: release the stage
					__syncwarp();
					if (lane == 0)
						mbar_arrive(&empty[s]);
				}
				__syncwarp();
				if (wide && k < full_groups) {
#pragma unroll
					for (int i = 0; i < kStores; ++i)
						*reinterpret_cast<uint4 *>(drow + i * store_step) =
							*reinterpret_cast<const uint4 *>(ld_addr + i * kStoreRows * kStageBytes);
				} else {
					for (int i = 0; i < kStores; ++i) {
						const int row = (g_begin + k) * 16 + st_row + i * kStoreRows;
						if (row < J.dst_h && st_col < J.dst_w) {
							const uint4 v = *reinterpret_cast<const uint4 *>(ld_addr + i * kStoreRows * kStageBytes);
							uint16_t *d = reinterpret_cast<uint16_t *>(dst + static_cast<ptrdiff_t>(row) * dst_stride) + st_col;
							if (J.vec_ok && st_col + 8 <= J.dst_w) {
								*reinterpret_cast<uint4 *>(d) = v;
							} else {
								const uint32_t w[4] = { v.x, v.y, v.z, v.w };
								for (int q = 0; q < 8 && st_col + q < J.dst_w; ++q)
									d[q] = static_cast<uint16_t>(w[q >> 1] >> (16 * (q & 1)));
							}
						}
					}
				}
				__syncwarp();
			} else {
				__syncwarp();
				if (lane == 0)
					mbar_arrive(&empty[s]);
			}
			prev_vb = vbk;
			drow += group_step;
			if (++s == NS) {
				s = 0;
				ph ^= 1;
			}
		}
	}
}

// An identity plane's rows g_begin*16 .. (g_begin + ngroups)*16 - 1, copied
// by every thread of the CTA, with no pipeline: a batch's identity
// conversions ride in the same launch. The job's src_w is the row length in
// bytes; vec_ok says whether planes, strides and rows allow 16-byte chunks.
__device__ __forceinline__ void copy_item(const FusedJob &J, int g_begin, int ngroups)
{
	const int row0 = g_begin * 16, row1 = min(J.dst_h, (g_begin + ngroups) * 16);
	const int row_bytes = J.src_w;
	const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	// one warp per row, its lanes along the row
	for (int r = row0 + warp; r < row1; r += warps) {
		const char *s = static_cast<const char *>(J.src) + static_cast<ptrdiff_t>(r) * J.src_stride;
		char *d = static_cast<char *>(J.dst) + static_cast<ptrdiff_t>(r) * J.dst_stride;
		if (J.vec_ok) {
			for (int c = lane * 16; c < row_bytes; c += 32 * 16)
				*reinterpret_cast<uint4 *>(d + c) = __ldg(reinterpret_cast<const uint4 *>(s + c));
		} else {
			for (int c = lane; c < row_bytes; c += 32)
				d[c] = s[c];
		}
	}
}

// Group bases of an item into shared memory (all threads).
__device__ __forceinline__ void load_bases(Pipe &p, const FusedJob &J, int g_begin, int ngroups)
{
	for (int g = threadIdx.x; g < ngroups; g += blockDim.x)
		p.vb[g] = __ldg(J.v_base + g_begin + g);
}

// Kernel for the jobs of one variant. The launch's (strip, 16-row group)
// units are numbered job by job and strip by strip. Without `ranges` each
// CTA takes an equal contiguous range of them; with it, CTA b takes the two
// ranges [ranges[4b], ranges[4b+1]) and [ranges[4b+2], ranges[4b+3]) in
// order (a whole strip, so that neighbouring CTAs run neighbouring strips in
// step and read their shared columns once through L2, then an equal share of
// the strips left over).
template <bool H_FIRST, int KV, int KH>
__global__ void __launch_bounds__(tma_threads(H_FIRST), 2)
chain_tma_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_items, const int *__restrict__ ranges,
                 const __grid_constant__ FusedJob single, const __grid_constant__ SmemLayout L,
                 const __grid_constant__ CUtensorMap single_map)
{
	extern __shared__ float4 smem4[];
	__shared__ int abort_item;
	Pipe p;
	pipe_init(p, smem4, L, &abort_item);
	int r_begin[2], r_end[2];
	if (ranges) {
		r_begin[0] = __ldg(ranges + 4 * blockIdx.x);
		r_end[0] = __ldg(ranges + 4 * blockIdx.x + 1);
		r_begin[1] = __ldg(ranges + 4 * blockIdx.x + 2);
		r_end[1] = __ldg(ranges + 4 * blockIdx.x + 3);
	} else {
		r_begin[0] = static_cast<int>(static_cast<long long>(blockIdx.x) * total_items / gridDim.x);
		r_end[0] = static_cast<int>(static_cast<long long>(blockIdx.x + 1) * total_items / gridDim.x);
		r_begin[1] = r_end[1] = 0;
	}
	for (int r = 0; r < 2 && !abort_item; ++r) {
		const int t_end = r_end[r];
		for (int t = r_begin[r]; t < t_end;) {
			const FusedJob &J = jobs ? jobs[find_job(jobs, num_jobs, t)] : single;
			const int local = t - J.item_begin;
			const int strip = local / J.groups;
			const int g_begin = local - strip * J.groups;
			const int ngroups = min(J.groups - g_begin, t_end - t);
			t += ngroups;
			load_bases(p, J, g_begin, ngroups);
			chain_item<H_FIRST, KV, KH, true>(p, L, J, jobs ? J.tmap : static_cast<const void *>(&single_map), strip,
			                                  g_begin, ngroups);
			p.base += ngroups;
			__syncthreads();  // the next item rewrites the group bases and the ring
			if (abort_item)
				break;
		}
	}
	pipe_finish(p);
}

// Variant codes of mixed launches: the chained kernel's variant - 200
// (H first, KV, KH), or kCopyVariant for an identity plane.
constexpr int kCopyVariant = 1000;

// One launch over a batch of mixed jobs: every chained variant and identity
// copies. CTAs take chunks of units from a counter (guided sizes, cut by the
// host from estimated costs: large chunks first, small ones last, so that
// the CTAs end together); an item is dispatched on its job's variant.
__global__ void __launch_bounds__(tma_threads(true), 2)
chain_mixed_kernel(const FusedJob *__restrict__ jobs, int num_jobs, const __grid_constant__ WorkChunks C,
                   const __grid_constant__ SmemLayout L)
{
	extern __shared__ float4 smem4[];
	__shared__ int abort_item;
	__shared__ int chunk;
	Pipe p;
	pipe_init(p, smem4, L, &abort_item);
	// chunks in the order CTAs ask for them (guided sizes: large first)
	for (;;) {
		const int m = next_chunk(C, &chunk);
		if (m < 0 || abort_item)
			break;
		const int t_end = __ldg(C.bounds + m + 1);
		for (int t = __ldg(C.bounds + m); t < t_end;) {
			const FusedJob &J = jobs[find_job(jobs, num_jobs, t)];
			const int local = t - J.item_begin;
			const int strip = local / J.groups;
			const int g_begin = local - strip * J.groups;
			const int ngroups = min(J.groups - g_begin, t_end - t);
			t += ngroups;
			const int v = J.variant;
			if (v == kCopyVariant) {
				copy_item(J, g_begin, ngroups);
			} else {
				load_bases(p, J, g_begin, ngroups);
				switch (v) {
#define ZG_CHAIN_CASE(HF, KV, KH)                                                                     \
	case (HF ? 12 : 0) + (KV - 1) * 4 + (KH - 1):                                                      \
		chain_item<HF, KV, KH, false>(p, L, J, J.tmap, strip, g_begin, ngroups);                     \
		break;
					ZG_CHAIN_CASE(true, 1, 1) ZG_CHAIN_CASE(true, 1, 2) ZG_CHAIN_CASE(true, 1, 3) ZG_CHAIN_CASE(true, 1, 4)
					ZG_CHAIN_CASE(true, 2, 1) ZG_CHAIN_CASE(true, 2, 2) ZG_CHAIN_CASE(true, 2, 3) ZG_CHAIN_CASE(true, 2, 4)
					ZG_CHAIN_CASE(true, 3, 1) ZG_CHAIN_CASE(true, 3, 2) ZG_CHAIN_CASE(true, 3, 3) ZG_CHAIN_CASE(true, 3, 4)
					ZG_CHAIN_CASE(false, 1, 1) ZG_CHAIN_CASE(false, 1, 2) ZG_CHAIN_CASE(false, 1, 3) ZG_CHAIN_CASE(false, 1, 4)
					ZG_CHAIN_CASE(false, 2, 1) ZG_CHAIN_CASE(false, 2, 2) ZG_CHAIN_CASE(false, 2, 3) ZG_CHAIN_CASE(false, 2, 4)
					ZG_CHAIN_CASE(false, 3, 1) ZG_CHAIN_CASE(false, 3, 2) ZG_CHAIN_CASE(false, 3, 3) ZG_CHAIN_CASE(false, 3, 4)
#undef ZG_CHAIN_CASE
				default:
					break;
				}
			}
			p.base += J.variant == kCopyVariant ? 0 : ngroups;
			__syncthreads();  // the next item rewrites the group bases and the ring
			if (abort_item)
				break;
		}
	}
	pipe_finish(p);
	chunks_finish(C);  // the last CTA out leaves the counter zero for the next launch
}

} // namespace chain_detail
} // namespace zg
