// Chained tensor-core u16 kernel, TMA pipeline form.
//
// Arithmetic, tiles and stores are those of chain_kernel.cuh. What differs is
// how source lines and tap fragments reach shared memory and how the warps
// stay in step:
//
//  - Source lines arrive as 2-D tensor copies (cp.async.bulk.tensor) of
//    16-line blocks of the strip's column window, the vertical tap fragments
//    of a group as one bulk copy. Block b of the plane lands in ring block
//    b mod NB, so line l sits in ring line l mod (16 NB) as in the cp.async
//    form; every block starts on a 128-byte boundary (16 lines x a pitch of
//    16 mod 32 bytes).
//  - A producer warp (one lane) issues the copies; the consumer warps only
//    compute. Group g of the CTA's pipeline uses stage s = g mod NS: a "full"
//    mbarrier whose transaction count covers the group's copies, and an
//    "empty" mbarrier on which each consumer warp arrives once it has read
//    the group. No CTA-wide barrier runs per group: the producer runs ahead
//    until a ring block or fragment slot it is about to overwrite is still
//    being read, and consumer warps drift apart as far as that allows.
//  - Source blocks wholly below the plane are not copied: the issuing thread
//    writes them as zero lines before it arrives on the group's barrier.
//  - Every mbarrier wait is bounded. A wait that runs out records its cause in
//    g_chain_pipeline_error, the CTA stops, and the issuing thread first waits
//    (again bounded) for the copies it still has in flight.
#pragma once

#include <cuda.h>

#include "chain_kernel.cuh"
#include "pipeline.cuh"

namespace zg {
namespace chain_detail {

constexpr int kBlockLines = 16;                     // source lines per tensor copy

// Nonzero after a pipeline wait ran out: 1 = group data never arrived, 2 = a
// buffer was never released, 3 = ring too small for one group (planner error).
__device__ int g_chain_pipeline_error;

// Kernel. Shared memory (SmemLayout, from a 128-byte aligned base): ring of
// NB = in_rows / kBlockLines blocks of source lines (in_off), NS = ring_rows
// slots of vertical tap fragments (vcoef_off), one staging tile pair per
// consumer warp (tile_off), the item's group bases (vbase_off), NS full and
// NS empty mbarriers (stage_off).
// Threads of a CTA: the consumer warps of the cp.async form plus one
// producer warp.
__host__ __device__ constexpr int tma_threads(bool h_first)
{
	return (warps_per_cta(h_first) + 1) * 32;
}

template <bool H_FIRST, int KV, int KH>
__global__ void __launch_bounds__(tma_threads(H_FIRST), H_FIRST ? 4 : 2)
chain_tma_kernel(const FusedJob *__restrict__ jobs, int num_jobs, int total_items, const __grid_constant__ FusedJob single,
                 const __grid_constant__ SmemLayout L, const __grid_constant__ CUtensorMap single_map)
{
	extern __shared__ float4 smem4[];
	__shared__ int abort_item;
	// tensor copies land on 128-byte boundaries: align the layout's base
	char *smem = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(smem4) + 127) & ~static_cast<uintptr_t>(127));
	char *ring = smem + L.in_off;
	char *vslots = smem + L.vcoef_off;
	int *vb = reinterpret_cast<int *>(smem + L.vbase_off);
	uint64_t *full = reinterpret_cast<uint64_t *>(smem + L.stage_off);
	const int NS = L.ring_rows;
	uint64_t *empty = full + NS;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	constexpr int kSlotBytes = KV * 2 * 32 * 16;
	constexpr int kTilesPerWarp = tiles_per_warp(KV, KH);
	constexpr int kWarps = warps_per_cta(H_FIRST);  // consumer warps; warp kWarps issues the copies
	constexpr int kThreads = tma_threads(H_FIRST);
	constexpr int kStripTiles = kWarps * kTilesPerWarp;
	const bool producer = warp == kWarps;
	char *stage = smem + L.tile_off + (producer ? 0 : warp) * kWarpStage;
	const int IR = L.in_rows;
	const int NB = IR / kBlockLines;
	const int P = L.pitch * 2;
	char *st_addr = stage + (((lane >> 4) << 3) + (lane & 7)) * kStageBytes + ((lane >> 3) & 1) * 16;
	constexpr int kStoreRows = kTilesPerWarp == 2 ? 8 : 16;
	constexpr int kStores = 16 / kStoreRows;
	const int st_row = kTilesPerWarp == 2 ? (lane >> 3) + 4 * ((lane >> 2) & 1)
	                                      : ((lane >> 3) & 1) + 8 * (lane >> 4) + 2 * ((lane >> 1) & 3);
	const int st_tile = kTilesPerWarp == 2 ? (lane >> 1) & 1 : 0;
	const char *ld_addr = stage + st_tile * kTileStage + st_row * kStageBytes + (lane & 1) * 16;

	if (threadIdx.x == 0) {
		for (int s = 0; s < NS; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], kWarps);
		}
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		abort_item = 0;
	}
	__syncthreads();

	// pipeline counters (groups since the kernel started): `base` is the
	// current item's first group; the producer also tracks `released` (groups
	// every consumer warp has finished, as observed on the empty barriers)
	// and `issued`
	unsigned base = 0, released = 0, issued = 0;
	int error = 0;

	const int t_end = static_cast<int>(static_cast<long long>(blockIdx.x + 1) * total_items / gridDim.x);
	for (int t = static_cast<int>(static_cast<long long>(blockIdx.x) * total_items / gridDim.x); t < t_end;) {
		const FusedJob *Jp = jobs ? &jobs[find_job(jobs, num_jobs, t)] : &single;
		const Item it = make_item(*Jp, t, t_end, kStripTiles, kThreads);
		t += it.g_end - it.g_begin;
		for (int g = it.g_begin + threadIdx.x; g < it.g_end; g += kThreads)
			vb[g - it.g_begin] = __ldg(Jp->v_base + g);
		const int ngroups = it.g_end - it.g_begin;

		if (producer) {
			__syncthreads();  // group bases visible; every warp is done with the previous item
			if (lane == 0 && !error) {
				const void *tmap = jobs ? Jp->tmap : static_cast<const void *>(&single_map);
				const char *vtab = reinterpret_cast<const char *>(Jp->v_dense);
				// next source block to load; first group of the item whose
				// window starts at or after the block being replaced
				int next_blk = vb[0] / kBlockLines;
				int gneed = 0;
				// advance `released` to n; false when a wait ran out
				auto release_to = [&](unsigned n) -> bool {
					while (released < n) {
						if (!mbar_wait(&empty[released % NS], (released / NS) & 1))
							return false;
						++released;
					}
					return true;
				};
				const int in_blks = (it.src_h + kBlockLines - 1) / kBlockLines;
				asm volatile("prefetch.tensormap [%0];\n" ::"l"(tmap) : "memory");
				for (int k = 0; k < ngroups; ++k) {
					const unsigned g = base + k;
					const int s = static_cast<int>(g % NS);
					// the stage's fragment slot was last read by group g - NS
					if (g >= static_cast<unsigned>(NS) && !release_to(g - NS + 1)) {
						error = 2;
						break;
					}
					const int last_blk = (vb[k] + 16 * KV - 1) / kBlockLines;
					for (int b = next_blk; b <= last_blk && !error; ++b) {
						// ring block b mod NB held block b - NB, which groups
						// read up to the first one whose window starts past it
						while (gneed < ngroups && vb[gneed] < (b - NB + 1) * kBlockLines)
							++gneed;
						if (gneed > k)
							error = 3;  // the ring cannot hold one window
						else if (!release_to(base + gneed))
							error = 2;
					}
					if (error)
						break;
					// blocks wholly below the plane (windows are padded to
					// 16 KV lines; their taps there are zero) become zero
					// lines, written here, not copied
					const int copy_end = min(last_blk + 1, in_blks);
					const int ncopy = max(0, copy_end - next_blk);
					for (int b = max(next_blk, in_blks); b <= last_blk; ++b) {
						float4 *z = reinterpret_cast<float4 *>(ring + (b % NB) * kBlockLines * P);
						for (int i = 0; i < kBlockLines * P / 16; ++i)
							z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
						// later tensor copies into this block come after these stores
						asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
					}
					mbar_arrive_expect_tx(&full[s], static_cast<unsigned>(kSlotBytes + ncopy * kBlockLines * P));
					for (int b = next_blk; b < copy_end; ++b)
						tma_load_2d(ring + (b % NB) * kBlockLines * P, tmap, it.xlo, b * kBlockLines, &full[s]);
					bulk_load(vslots + s * kSlotBytes, vtab + static_cast<size_t>(it.g_begin + k) * kSlotBytes,
					          kSlotBytes, &full[s]);
					next_blk = max(next_blk, last_blk + 1);
					issued = g + 1;
				}
				if (error)
					abort_item = 1;  // benign race: every writer stores 1
			}
		} else {
			const int ntiles = (it.dst_w + kTileW - 1) / kTileW;
			const int tile0 = it.strip * kStripTiles + warp * kTilesPerWarp;
			uint4 ah[kTilesPerWarp][KH][2];
			int rel[kTilesPerWarp];
			Carry carry[kTilesPerWarp];
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
			__syncthreads();  // group bases visible; every warp is done with the previous item

			int cur_vb = vb[0];
			int cur_slot = wrap(cur_vb % IR, IR);
			const bool active = tile0 * kTileW < it.dst_w;
			for (int k = 0; k < ngroups; ++k) {
				const unsigned g = base + k;
				const int s = static_cast<int>(g % NS);
				// every lane polls; the warp goes on only when all saw the copies land
				if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (g / NS) & 1))) {
					error = 1;
					abort_item = 1;  // benign race: every writer stores 1
					break;
				}
				const int vbk = vb[k];
				const bool reuse = H_FIRST && KV == 1 && k > 0 && vbk - cur_vb == 8;
				cur_slot = wrap(cur_slot + (vbk - cur_vb), IR);
				cur_vb = vbk;
				if (active) {
					const uint4 *avs = reinterpret_cast<const uint4 *>(vslots + s * kSlotBytes) + lane;
					uint4 av[KV][2];
#pragma unroll
					for (int kv = 0; kv < KV; ++kv) {
						av[kv][0] = avs[(kv * 2 + 0) * 32];
						av[kv][1] = avs[(kv * 2 + 1) * 32];
					}
					uint32_t m[kTilesPerWarp][4];
#pragma unroll
					for (int j = 0; j < kTilesPerWarp; ++j)
						tile_compute<H_FIRST, KV, KH>(it, ring, IR, P, cur_slot, rel[j], ah[j], av, carry[j], reuse, m[j]);
					// the group's shared data are in registers: release the stage
					__syncwarp();
					if (lane == 0)
						mbar_arrive(&empty[s]);
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
				} else {
					__syncwarp();
					if (lane == 0)
						mbar_arrive(&empty[s]);
				}
				drow += group_step;
			}
		}
		base += ngroups;
		__syncthreads();  // the next item rewrites the group bases and the ring
		if (abort_item)
			break;
	}

	if (producer && lane == 0 && (error || abort_item)) {
		atomicExch(&g_chain_pipeline_error, error ? error : 1);
		// copies still in flight land before the CTA leaves: only the last NS
		// issued groups can have any (an earlier group's stage was reissued
		// only after every consumer had read it)
		for (unsigned g = issued > static_cast<unsigned>(NS) ? issued - NS : 0; g < issued; ++g)
			mbar_wait(&full[g % NS], (g / NS) & 1);
	} else if (!producer && lane == 0 && error) {
		atomicExch(&g_chain_pipeline_error, error);
	}
}

} // namespace chain_detail
} // namespace zg
