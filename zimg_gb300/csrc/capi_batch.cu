// C ABI: batches of conversions over planes of uneven sizes.
//
// Fused jobs are grouped by kernel variant; each group runs as ONE persistent
// launch over the concatenated tile lists of its jobs (a device table of
// FusedJob entries, one per plane). Identity conversions are copied by one
// batched copy launch. Jobs that cannot be fused (wide filters, single
// passes) run through their own conversion.
#include "capi_common.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <string>

using namespace zg;

struct zg_batch {
	struct Group {
		int variant;
		SmemLayout layout;
		int grid;
		int first;  // first entry in the device job table
		int count;
		int tiles;
		// chained groups: the TMA-pipelined kernel, when every source plane
		// of the group has a tensor map (decided at each io upload)
		bool tma_plan = false;
		bool tma_now = false;
		SmemLayout tlayout{};
		int tgrid = 0;
		int ranges_off = -1;  // CTA unit ranges in ranges_dev (ints), or -1
		// guided chunks (CUDA-core streaming groups): bounds at chunks_off in
		// chunks_dev, num_chunks chunks, the counter pair at `sched` in
		// sched_dev; num_chunks 0: a static split (the chained groups keep
		// strips in step, measured faster for them)
		int chunks_off = 0, num_chunks = 0, sched = 0;
	};

	int device;
	std::vector<zg_resize *> jobs;
	std::vector<int> table_index;  // per job: entry in the fused table, or -1
	std::vector<size_t> tmp_offset;
	size_t tmp_size = 0;
	std::vector<zg_batch_io> io;
	std::vector<Group> groups;
	std::vector<int> ranges_host;
	DeviceBuffer ranges_dev;
	std::vector<int> chunks_host;
	DeviceBuffer chunks_dev;
	DeviceBuffer sched_dev;  // two words per group (zero between launches)
	std::vector<FusedJob> table_host;
	DeviceBuffer table_dev;
	std::vector<CUtensorMap> maps_host;  // per table entry (chained TMA groups)
	DeviceBuffer maps_dev;
	// identity conversions: one batched copy launch
	std::vector<int> copy_jobs;
	std::vector<PlaneCopy> copy_host;
	DeviceBuffer copy_dev;
	unsigned long long copy_chunks = 0;
	// one launch for the chained groups and the identity copies together
	// (chain_mixed_kernel), when every chained job's source plane has a
	// tensor map: its own job table, tensor maps and per-CTA unit ranges
	bool mixed_plan = false;
	bool mixed_now = false;
	SmemLayout mixed_layout{};
	int mixed_grid = 0;
	std::vector<int> mixed_jobs;        // batch job of each mixed table entry
	std::vector<FusedJob> mixed_host;
	DeviceBuffer mixed_dev;
	std::vector<CUtensorMap> mixed_maps_host;
	DeviceBuffer mixed_maps_dev;
	DeviceBuffer mixed_ranges_dev;      // chunk bounds (mixed_chunks + 1 unit indices)
	int mixed_chunks = 0;
	DeviceBuffer mixed_sched_dev;       // the launch's chunk counter and CTA exit count (zero between launches)
	cudaGraphExec_t graph = nullptr;
	cudaStream_t graph_stream = nullptr;
	void *graph_tmp = nullptr;
	// independent launches (variant groups, the copy launch, unfused jobs) run
	// concurrently on side streams forked from and joined to the caller's
	mutable std::vector<cudaStream_t> side;
	mutable std::vector<cudaEvent_t> joins;
	mutable cudaEvent_t fork = nullptr;

	~zg_batch()
	{
		if (graph)
			cudaGraphExecDestroy(graph);
		for (cudaStream_t s : side)
			cudaStreamDestroy(s);
		for (cudaEvent_t e : joins)
			cudaEventDestroy(e);
		if (fork)
			cudaEventDestroy(fork);
		for (auto *j : jobs)
			zg_resize_free(j);
	}
};

namespace {

void rethrow_last(zg_error_code rc)
{
	char msg[256];
	zg_get_last_error(msg, sizeof(msg));
	throw Error(rc, msg);
}

constexpr size_t kSideStreams = 4;

// CUDA-core streaming launches take guided chunks of their units (false
// when the environment sets ZG_BATCH_CHUNKS=0: equal static shares).
bool batch_chunks_enabled()
{
	static const bool on = [] {
		const char *e = std::getenv("ZG_BATCH_CHUNKS");
		return !(e && e[0] == '0');
	}();
	return on;
}

void batch_launch(const zg_batch *b, void *tmp, cudaStream_t st)
{
	if (b->io.size() != b->jobs.size())
		throw Error(kErrLogic, "zg_batch_set_io was not called");
	const FusedJob *table = static_cast<const FusedJob *>(b->table_dev.get());
	std::vector<std::function<void(cudaStream_t)>> work;
	if (b->mixed_now) {
		work.push_back([b](cudaStream_t s) {
			WorkChunks c;
			c.bounds = static_cast<const int *>(b->mixed_ranges_dev.get());
			c.num = b->mixed_chunks;
			c.sched = static_cast<unsigned *>(b->mixed_sched_dev.get());
			cuda_check(launch_chain_mixed(static_cast<const FusedJob *>(b->mixed_dev.get()),
			                              static_cast<int>(b->mixed_host.size()), c, b->mixed_layout, b->mixed_grid, s),
			           "mixed batch launch");
		});
	}
	for (const auto &g : b->groups) {
		if (b->mixed_now && g.tma_plan)
			continue;  // in the mixed launch
		const int *ranges = g.ranges_off < 0 ? nullptr : static_cast<const int *>(b->ranges_dev.get()) + g.ranges_off;
		WorkChunks c;
		if (!g.tma_now && g.num_chunks > 0) {
			c.bounds = static_cast<const int *>(b->chunks_dev.get()) + g.chunks_off;
			c.num = g.num_chunks;
			c.sched = static_cast<unsigned *>(b->sched_dev.get()) + g.sched;
		}
		work.push_back([&g, table, ranges, c](cudaStream_t s) {
			FusedJob unused{};
			if (g.tma_now)
				cuda_check(launch_chain_tma(g.variant, table + g.first, g.count, g.tiles, ranges, g.tlayout, g.tgrid,
				                            unused, nullptr, s),
				           "fused batch launch");
			else
				cuda_check(launch_fused(g.variant, table + g.first, g.count, g.tiles, g.layout, g.grid, unused, s, c),
				           "fused batch launch");
		});
	}
	if (!b->copy_jobs.empty() && !b->mixed_now) {
		work.push_back([b](cudaStream_t s) {
			cuda_check(launch_plane_copies(static_cast<const PlaneCopy *>(b->copy_dev.get()),
			                               static_cast<int>(b->copy_jobs.size()), b->copy_chunks, s),
			           "batch plane copies");
		});
	}
	for (size_t i = 0; i < b->jobs.size(); ++i) {
		if (b->table_index[i] >= 0 || b->jobs[i]->num_passes == 0)
			continue;
		work.push_back([b, i, tmp](cudaStream_t s) {
			const zg_batch_io &io = b->io[i];
			void *t = b->tmp_size ? static_cast<char *>(tmp) + b->tmp_offset[i] : nullptr;
			zg_error_code rc = zg_resize_process(b->jobs[i], io.src, io.src_stride, io.dst, io.dst_stride, t,
			                                     reinterpret_cast<zg_stream>(s));
			if (rc != ZG_ERROR_SUCCESS)
				rethrow_last(rc);
		});
	}
	if (work.size() <= 1) {
		for (auto &w : work)
			w(st);
		return;
	}
	const size_t n = std::min(work.size(), kSideStreams);
	while (b->side.size() < n) {
		cudaStream_t s = nullptr;
		cudaEvent_t e = nullptr;
		cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "side stream");
		b->side.push_back(s);
		cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
		b->joins.push_back(e);
	}
	if (!b->fork)
		cuda_check(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "event");
	cuda_check(cudaEventRecord(b->fork, st), "fork");
	for (size_t k = 0; k < n; ++k)
		cuda_check(cudaStreamWaitEvent(b->side[k], b->fork, 0), "fork");
	for (size_t i = 0; i < work.size(); ++i)
		work[i](b->side[i % n]);
	for (size_t k = 0; k < n; ++k) {
		cuda_check(cudaEventRecord(b->joins[k], b->side[k]), "join");
		cuda_check(cudaStreamWaitEvent(st, b->joins[k], 0), "join");
	}
}

// Jobs whose fused plans have identical tables (the same conversion for many
// frames, as zimg runs one graph over a stream of frames) read one device copy
// of them: the first such job's. A launch then touches each distinct table
// once, and it stays in L2 instead of being fetched again per job.
void share_tables(zg_batch *b)
{
	std::map<std::pair<int, size_t>, std::vector<unsigned>> firsts;  // (variant, blob size) -> jobs owning a copy
	for (unsigned i = 0; i < b->jobs.size(); ++i) {
		zg_resize *r = b->jobs[i];
		if (!r->fused || r->fplan.blob.empty())
			continue;
		fused_bind(r->fplan, r->fblob.get());
		auto &cands = firsts[{ r->fplan.variant, r->fplan.blob.size() }];
		bool shared = false;
		for (unsigned f : cands) {
			const FusedPlan &q = b->jobs[f]->fplan;
			if (std::memcmp(q.blob.data(), r->fplan.blob.data(), q.blob.size()) == 0) {
				fused_bind(r->fplan, b->jobs[f]->fblob.get());
				shared = true;
				break;
			}
		}
		if (!shared)
			cands.push_back(i);
	}
}

// Estimated cost of one work unit of a mixed launch, in bytes at full HBM
// speed: the unit's share of its plane's algorithmic bytes over the fraction
// of the HBM roofline its kind of work reaches alone on GB300: H-first groups
// that reuse the previous group's products (2x upscales) ~70 %, other H-first
// groups ~38 %, V-first downscales ~47 %, identity copies ~90 %.
double unit_cost(const zg_resize *r, const FusedJob &j, bool copy)
{
	const double bpe = bytes_of(r->sample);
	const double bytes = (static_cast<double>(r->params.src_width) * r->params.src_height +
	                      static_cast<double>(r->params.dst_width) * r->params.dst_height) * bpe;
	const double units = std::max(1, fused_items(j));
	double eff = 0.9;
	if (!copy) {
		const bool hf = j.variant >= 12;
		const double reuse = r->fplan.reuse_frac;
		eff = hf ? 1.0 / (reuse / 0.70 + (1.0 - reuse) / 0.38) : 0.47;
	}
	return bytes / units / eff;
}

// The mixed launch (chain_mixed_kernel): every chained group whose layout
// admits the TMA form and every identity copy in one persistent launch, the
// units of each CTA balanced by estimated cost. Decided per plan here; used
// when every source plane also has a tensor map (upload_io).
void plan_mixed(zg_batch *b)
{
	b->mixed_plan = false;
	b->mixed_now = false;
	b->mixed_jobs.clear();
	b->mixed_host.clear();
	b->mixed_dev.release();
	b->mixed_maps_dev.release();
	b->mixed_ranges_dev.release();
	b->mixed_sched_dev.release();
	b->mixed_chunks = 0;
	if (!chain_tma_enabled())
		return;
	std::vector<const FusedPlan *> plans;
	int chained_groups = 0;
	for (const auto &g : b->groups) {
		if (!g.tma_plan)
			continue;
		++chained_groups;
		for (int e = g.first; e < g.first + g.count; ++e) {
			for (size_t i = 0; i < b->jobs.size(); ++i)
				if (b->table_index[i] == e) {
					plans.push_back(&b->jobs[i]->fplan);
					b->mixed_jobs.push_back(static_cast<int>(i));
				}
		}
	}
	// worth one launch when it replaces more than one
	if (plans.empty() || chained_groups + (b->copy_jobs.empty() ? 0 : 1) < 2 ||
	    !chain_tma_layout(plans.data(), static_cast<int>(plans.size()), &b->mixed_layout)) {
		b->mixed_jobs.clear();
		return;
	}
	for (int c : b->copy_jobs)
		b->mixed_jobs.push_back(c);
	std::vector<double> cost;
	int units = 0;
	for (size_t e = 0; e < b->mixed_jobs.size(); ++e) {
		const zg_resize *r = b->jobs[b->mixed_jobs[e]];
		FusedJob j{};
		const bool copy = r->num_passes == 0;
		if (copy) {
			j.variant = chain_mixed_copy_variant();
			j.src_w = static_cast<int>(r->params.dst_width * bytes_of(r->sample));
			j.dst_w = static_cast<int>(r->params.dst_width);
			j.dst_h = static_cast<int>(r->params.dst_height);
			j.groups = (j.dst_h + 15) / 16;
			j.strips = 1;
			j.segments = j.groups;
		} else {
			j = r->fplan.job;
		}
		j.item_begin = units;
		units += fused_items(j);
		cost.push_back(unit_cost(r, j, copy));
		b->mixed_host.push_back(j);
	}
	b->mixed_grid = std::min(chain_mixed_grid_size(static_cast<size_t>(b->mixed_layout.total_bytes)), units);
	// guided chunks of the units by estimated cost, at least 12 units each;
	// chained jobs' chunks end on strip boundaries where that moves the end
	// by at most a quarter (an item's start costs about 3 groups), identity
	// copies (last in the table) anywhere
	std::vector<int> item_begin, items, strip_units;
	for (const FusedJob &j : b->mixed_host) {
		item_begin.push_back(j.item_begin);
		items.push_back(fused_items(j));
		strip_units.push_back(j.variant == chain_mixed_copy_variant() ? 0 : j.groups);
	}
	const std::vector<int> bounds = chain_mixed_chunks(item_begin, items, cost, strip_units, b->mixed_grid, 12);
	if (bounds.size() < 2) {
		b->mixed_jobs.clear();
		b->mixed_host.clear();
		return;
	}
	b->mixed_chunks = static_cast<int>(bounds.size()) - 1;
	b->mixed_ranges_dev.reset(bounds.size() * sizeof(int));
	cuda_check(cudaMemcpy(b->mixed_ranges_dev.get(), bounds.data(), bounds.size() * sizeof(int), cudaMemcpyHostToDevice),
	           "mixed batch chunks");
	b->mixed_sched_dev.reset(2 * sizeof(unsigned));
	cuda_check(cudaMemset(b->mixed_sched_dev.get(), 0, 2 * sizeof(unsigned)), "mixed batch chunks");
	b->mixed_dev.reset(b->mixed_host.size() * sizeof(FusedJob));
	b->mixed_maps_host.assign(b->mixed_host.size(), CUtensorMap{});
	b->mixed_maps_dev.reset(b->mixed_host.size() * sizeof(CUtensorMap));
	b->mixed_plan = true;
}

// Tmp offsets, fused work segmentation and the persistent launch groups
// (fused jobs grouped by kernel variant, in job order within a group).
void regroup(zg_batch *b)
{
	const unsigned num_jobs = static_cast<unsigned>(b->jobs.size());
	b->tmp_offset.clear();
	b->tmp_size = 0;
	for (unsigned i = 0; i < num_jobs; ++i) {
		b->tmp_offset.push_back(b->tmp_size);
		if (!b->jobs[i]->fused)
			b->tmp_size += (b->jobs[i]->tmp_size + 255) & ~static_cast<size_t>(255);
	}
	b->groups.clear();
	b->ranges_host.clear();
	b->chunks_host.clear();
	b->table_host.clear();
	b->table_dev.release();
	share_tables(b);
	// one wave of work items across the whole batch: split strips into row
	// segments only as far as needed to fill the GPU
	std::vector<FusedPlan *> all;
	for (unsigned i = 0; i < num_jobs; ++i)
		if (b->jobs[i]->fused)
			all.push_back(&b->jobs[i]->fplan);
	if (!all.empty())
		fused_segment(all.data(), static_cast<int>(all.size()), fused_wave_items());

	// group fused jobs by variant, in job order within a group
	std::map<int, std::vector<unsigned>> by_variant;
	for (unsigned i = 0; i < num_jobs; ++i)
		if (b->jobs[i]->fused)
			by_variant[b->jobs[i]->fplan.variant].push_back(i);
	b->table_index.assign(num_jobs, -1);
	for (auto &kv : by_variant) {
		zg_batch::Group g{ kv.first, SmemLayout{}, 0, static_cast<int>(b->table_host.size()), 0, 0 };
		std::vector<const FusedPlan *> plans;
		for (unsigned i : kv.second) {
			FusedJob j = b->jobs[i]->fplan.job;
			j.item_begin = g.tiles;
			g.tiles += fused_items(j);
			plans.push_back(&b->jobs[i]->fplan);
			b->table_index[i] = static_cast<int>(b->table_host.size());
			b->table_host.push_back(j);
			++g.count;
		}
		g.layout = fused_layout(plans.data(), static_cast<int>(plans.size()));
		g.grid = fused_grid_size(g.variant, static_cast<size_t>(g.layout.total_bytes));
		if (plans[0]->chain && chain_tma_enabled()) {
			g.tma_plan = chain_tma_layout(plans.data(), static_cast<int>(plans.size()), &g.tlayout);
			if (g.tma_plan) {
				g.tgrid = chain_tma_grid_size(g.variant, static_cast<size_t>(g.tlayout.total_bytes));
				// jobs of one shape with at least a strip per CTA: strips in
				// step across neighbouring CTAs
				bool same = true;
				for (unsigned i : kv.second)
					same = same && b->jobs[i]->fplan.job.groups == b->jobs[kv.second[0]]->fplan.job.groups;
				const char *order = std::getenv("ZG_CHAIN_ORDER");
				const bool lockstep = !(order && std::string(order) == "equal");
				const std::vector<int> r = same && lockstep ? chain_tma_lockstep_ranges(
				                                                  g.tiles, b->jobs[kv.second[0]]->fplan.job.groups, g.tgrid)
				                                            : std::vector<int>();
				if (!r.empty()) {
					g.ranges_off = static_cast<int>(b->ranges_host.size());
					b->ranges_host.insert(b->ranges_host.end(), r.begin(), r.end());
				}
			}
		}
		// CUDA-core streaming groups: guided chunks of the group's units (cost
		// per unit: the job's samples over its units), ending on strip
		// boundaries where that moves the end by at most a quarter (measured:
		// bicubic 1.293 -> 1.214 ms per step)
		if (batch_chunks_enabled() && fused_takes_chunks(g.variant)) {
			std::vector<int> item_begin, items, strips_of;
			std::vector<double> cost;
			for (unsigned i : kv.second) {
				const FusedJob &j = b->table_host[b->table_index[i]];
				const zg_resize *r = b->jobs[i];
				item_begin.push_back(j.item_begin);
				items.push_back(fused_items(j));
				cost.push_back((static_cast<double>(r->params.src_width) * r->params.src_height +
				                static_cast<double>(r->params.dst_width) * r->params.dst_height) /
				               std::max(1, fused_items(j)));
				strips_of.push_back(j.segments);
			}
			const std::vector<int> bo = chain_mixed_chunks(item_begin, items, cost, strips_of, g.grid, 8);
			if (bo.size() >= 2) {
				g.chunks_off = static_cast<int>(b->chunks_host.size());
				g.num_chunks = static_cast<int>(bo.size()) - 1;
				g.sched = 2 * static_cast<int>(b->groups.size());
				b->chunks_host.insert(b->chunks_host.end(), bo.begin(), bo.end());
			}
		}
		b->groups.push_back(g);
	}
	b->chunks_dev.release();
	b->sched_dev.release();
	if (!b->chunks_host.empty()) {
		b->chunks_dev.reset(b->chunks_host.size() * sizeof(int));
		cuda_check(cudaMemcpy(b->chunks_dev.get(), b->chunks_host.data(), b->chunks_host.size() * sizeof(int),
		                      cudaMemcpyHostToDevice),
		           "work chunks");
		b->sched_dev.reset(2 * b->groups.size() * sizeof(unsigned));
		cuda_check(cudaMemset(b->sched_dev.get(), 0, 2 * b->groups.size() * sizeof(unsigned)), "work chunks");
	}
	b->ranges_dev.release();
	if (!b->ranges_host.empty()) {
		b->ranges_dev.reset(b->ranges_host.size() * sizeof(int));
		cuda_check(cudaMemcpy(b->ranges_dev.get(), b->ranges_host.data(), b->ranges_host.size() * sizeof(int),
		                      cudaMemcpyHostToDevice),
		           "strip ranges");
	}
	if (!b->table_host.empty()) {
		b->table_dev.reset(b->table_host.size() * sizeof(FusedJob));
		b->maps_host.assign(b->table_host.size(), CUtensorMap{});
		b->maps_dev.reset(b->table_host.size() * sizeof(CUtensorMap));
	}
	b->copy_jobs.clear();
	for (unsigned i = 0; i < num_jobs; ++i)
		if (b->jobs[i]->num_passes == 0)
			b->copy_jobs.push_back(static_cast<int>(i));
	b->copy_host.assign(b->copy_jobs.size(), PlaneCopy{});
	b->copy_dev.release();
	if (!b->copy_jobs.empty())
		b->copy_dev.reset(b->copy_jobs.size() * sizeof(PlaneCopy));
	plan_mixed(b);
}

// Plane pointers of the fused jobs into the device table (ordered on st; the
// host copy stays valid until the next upload, which waits for this one).
void upload_io(zg_batch *b, cudaStream_t st)
{
	for (size_t i = 0; i < b->jobs.size(); ++i) {
		if (b->table_index[i] >= 0) {
			const zg_batch_io &x = b->io[i];
			fused_set_io(b->table_host[b->table_index[i]], x.src, x.src_stride, x.dst, x.dst_stride);
		}
	}
	b->copy_chunks = 0;
	for (size_t c = 0; c < b->copy_jobs.size(); ++c) {
		const zg_resize *r = b->jobs[b->copy_jobs[c]];
		const zg_batch_io &x = b->io[b->copy_jobs[c]];
		PlaneCopy &p = b->copy_host[c];
		p.src = x.src;
		p.src_stride = x.src_stride;
		p.dst = x.dst;
		p.dst_stride = x.dst_stride;
		p.row_bytes = r->params.dst_width * bytes_of(r->sample);
		p.rows = r->params.dst_height;
		auto al = [](const void *q, ptrdiff_t s, unsigned a) {
			return reinterpret_cast<uintptr_t>(q) % a == 0 && s % a == 0;
		};
		const bool v16 = al(x.src, x.src_stride, 16) && al(x.dst, x.dst_stride, 16) && p.row_bytes % 16 == 0;
		const bool v4 = al(x.src, x.src_stride, 4) && al(x.dst, x.dst_stride, 4) && p.row_bytes % 4 == 0;
		p.unit = v16 ? 16 : (v4 ? 4 : 2);
		p.chunks_per_row = p.row_bytes / p.unit;
		p.chunk_begin = b->copy_chunks;
		b->copy_chunks += static_cast<unsigned long long>(p.chunks_per_row) * p.rows;
	}
	// tensor maps of the chained groups' source planes
	bool any_map = false;
	for (auto &g : b->groups) {
		g.tma_now = g.tma_plan;
		for (int e = g.first; g.tma_now && e < g.first + g.count; ++e)
			g.tma_now = chain_tma_source_map(&b->maps_host[e], b->table_host[e], g.tlayout);
		for (int e = g.first; e < g.first + g.count; ++e)
			b->table_host[e].tmap = g.tma_now ? static_cast<const CUtensorMap *>(b->maps_dev.get()) + e : nullptr;
		any_map = any_map || g.tma_now;
	}
	if (any_map)
		cuda_check(cudaMemcpyAsync(b->maps_dev.get(), b->maps_host.data(), b->maps_host.size() * sizeof(CUtensorMap),
		                           cudaMemcpyHostToDevice, st),
		           "batch io upload");
	// the mixed launch: plane pointers, tensor maps of the chained entries
	b->mixed_now = b->mixed_plan;
	for (size_t e = 0; b->mixed_now && e < b->mixed_host.size(); ++e) {
		const int i = b->mixed_jobs[e];
		const zg_batch_io &x = b->io[i];
		FusedJob &j = b->mixed_host[e];
		if (j.variant == chain_mixed_copy_variant()) {
			j.src = x.src;
			j.src_stride = x.src_stride;
			j.dst = x.dst;
			j.dst_stride = x.dst_stride;
			auto al = [](const void *q, ptrdiff_t sd) { return reinterpret_cast<uintptr_t>(q) % 16 == 0 && sd % 16 == 0; };
			j.vec_ok = al(x.src, x.src_stride) && al(x.dst, x.dst_stride) && j.src_w % 16 == 0;
			j.tmap = nullptr;
		} else {
			fused_set_io(j, x.src, x.src_stride, x.dst, x.dst_stride);
			b->mixed_now = chain_tma_source_map(&b->mixed_maps_host[e], j, b->mixed_layout);
			j.tmap = static_cast<const CUtensorMap *>(b->mixed_maps_dev.get()) + e;
		}
	}
	if (b->mixed_now) {
		cuda_check(cudaMemcpyAsync(b->mixed_maps_dev.get(), b->mixed_maps_host.data(),
		                           b->mixed_maps_host.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, st),
		           "batch io upload");
		cuda_check(cudaMemcpyAsync(b->mixed_dev.get(), b->mixed_host.data(), b->mixed_host.size() * sizeof(FusedJob),
		                           cudaMemcpyHostToDevice, st),
		           "batch io upload");
	}
	if (!b->copy_host.empty())
		cuda_check(cudaMemcpyAsync(b->copy_dev.get(), b->copy_host.data(), b->copy_host.size() * sizeof(PlaneCopy),
		                           cudaMemcpyHostToDevice, st), "batch io upload");
	if (!b->table_host.empty())
		cuda_check(cudaMemcpyAsync(b->table_dev.get(), b->table_host.data(), b->table_host.size() * sizeof(FusedJob),
		                           cudaMemcpyHostToDevice, st), "batch io upload");
	if (!b->table_host.empty() || !b->copy_host.empty())
		cuda_check(cudaStreamSynchronize(st), "batch io upload");
}

// How a conversion runs, for the autotuner's de-duplication of candidates.
int plan_mode(const zg_resize *r)
{
	if (r->num_passes == 0)
		return -1;
	return r->fused ? (r->fplan.mma ? 2 : 1) : (r->tensor_passes ? 3 : 0);
}

} // namespace

extern "C" {

zg_error_code zg_batch_create(const zg_resize_params *jobs, unsigned num_jobs, zg_batch **out)
{
	return guarded([&] {
		if (!jobs || !out || !num_jobs)
			throw Error(kErrIllegalArgument, "empty batch");
		*out = nullptr;
		auto b = std::make_unique<zg_batch>();
		b->device = current_device();
		for (unsigned i = 0; i < num_jobs; ++i) {
			zg_resize *r = nullptr;
			zg_error_code rc = zg_resize_create(&jobs[i], &r);
			if (rc != ZG_ERROR_SUCCESS)
				rethrow_last(rc);
			b->jobs.push_back(r);
		}

		regroup(b.get());
		*out = b.release();
	});
}

void zg_batch_free(zg_batch *b)
{
	delete b;
}

zg_error_code zg_batch_get_tmp_size(const zg_batch *b, size_t *out)
{
	return guarded([&] {
		if (!b || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		*out = b->tmp_size;
	});
}

zg_error_code zg_batch_set_io(zg_batch *b, const zg_batch_io *io, zg_stream stream)
{
	return guarded([&] {
		if (!b || !io)
			throw Error(kErrIllegalArgument, "null pointer");
		if (current_device() != b->device)
			throw Error(kErrLogic, "batch used on a different device than the one it was created on");
		for (size_t i = 0; i < b->jobs.size(); ++i) {
			const zg_resize_params &q = b->jobs[i]->params;
			const unsigned bpe = bytes_of(b->jobs[i]->sample);
			if (!io[i].src || !io[i].dst)
				throw Error(kErrIllegalArgument, "null plane pointer in batch io");
			if (abs_stride(io[i].src_stride) < static_cast<ptrdiff_t>(q.src_width * bpe) ||
			    abs_stride(io[i].dst_stride) < static_cast<ptrdiff_t>(q.dst_width * bpe))
				throw Error(kErrIllegalArgument, "stride smaller than a line in batch io");
			if (reinterpret_cast<uintptr_t>(io[i].src) % bpe || reinterpret_cast<uintptr_t>(io[i].dst) % bpe ||
			    io[i].src_stride % bpe || io[i].dst_stride % bpe)
				throw Error(kErrIllegalArgument, "batch io not aligned to the sample size");
		}
		b->io.assign(io, io + b->jobs.size());
		upload_io(b, reinterpret_cast<cudaStream_t>(stream));
		if (b->graph) {
			cudaGraphExecDestroy(b->graph);
			b->graph = nullptr;
		}
	});
}

zg_error_code zg_batch_process(const zg_batch *b, void *tmp, zg_stream stream)
{
	return guarded([&] {
		if (!b)
			throw Error(kErrIllegalArgument, "null pointer");
		if (b->tmp_size && !tmp)
			throw Error(kErrIllegalArgument, "tmp buffer required (zg_batch_get_tmp_size)");
		batch_launch(b, tmp, reinterpret_cast<cudaStream_t>(stream));
	});
}

zg_error_code zg_batch_process_graph(zg_batch *b, void *tmp, zg_stream stream)
{
	return guarded([&] {
		if (!b)
			throw Error(kErrIllegalArgument, "null pointer");
		if (b->tmp_size && !tmp)
			throw Error(kErrIllegalArgument, "tmp buffer required (zg_batch_get_tmp_size)");
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		if (!b->graph || b->graph_stream != st || b->graph_tmp != tmp) {
			if (b->graph) {
				cudaGraphExecDestroy(b->graph);
				b->graph = nullptr;
			}
			cudaStream_t cap = nullptr;
			cuda_check(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "stream");
			cudaGraph_t g = nullptr;
			cuda_check(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "begin capture");
			try {
				batch_launch(b, tmp, cap);
			} catch (...) {
				cudaStreamEndCapture(cap, &g);
				if (g)
					cudaGraphDestroy(g);
				cudaStreamDestroy(cap);
				throw;
			}
			cuda_check(cudaStreamEndCapture(cap, &g), "end capture");
			cudaStreamDestroy(cap);
			cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
			cudaGraphDestroy(g);
			cuda_check(e, "graph instantiate");
			b->graph_stream = st;
			b->graph_tmp = tmp;
		}
		cuda_check(cudaGraphLaunch(b->graph, st), "graph launch");
	});
}

zg_error_code zg_batch_autotune(zg_batch *b, zg_stream stream, unsigned *changed)
{
	return guarded([&] {
		if (!b)
			throw Error(kErrIllegalArgument, "null pointer");
		if (b->io.size() != b->jobs.size())
			throw Error(kErrLogic, "zg_batch_set_io was not called");
		if (current_device() != b->device)
			throw Error(kErrLogic, "batch used on a different device than the one it was created on");
		cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
		unsigned n_changed = 0;

		// jobs with identical parameters are tuned once, on up to kSample of their
		// planes; a plan replaces the static one only when it is kMargin faster
		constexpr size_t kSample = 16;
		constexpr int kReps = 2;
		constexpr float kMargin = 0.95f;
		std::vector<bool> done(b->jobs.size(), false);
		for (size_t i = 0; i < b->jobs.size(); ++i) {
			if (done[i])
				continue;
			const zg_resize_params &q = b->jobs[i]->params;
			std::vector<size_t> same;
			for (size_t j = i; j < b->jobs.size(); ++j) {
				if (!done[j] && std::memcmp(&b->jobs[j]->params, &q, sizeof(q)) == 0) {
					same.push_back(j);
					done[j] = true;
				}
			}
			if (q.engine != ZG_ENGINE_AUTO || !q.allow_fusion || plan_mode(b->jobs[i]) < 0)
				continue;

			// candidates: every distinct way the planner can run this conversion
			struct Cand {
				zg_resize *r;
				float ms;
			};
			std::vector<Cand> cands;
			const zg_engine engines[3] = { ZG_ENGINE_CUDA, ZG_ENGINE_CUDA, ZG_ENGINE_TENSOR };
			const int fusion[3] = { 1, 0, 1 };
			for (int c = 0; c < 3; ++c) {
				zg_resize_params p = q;
				p.engine = engines[c];
				p.allow_fusion = fusion[c];
				zg_resize *r = nullptr;
				if (zg_error_code rc = zg_resize_create(&p, &r))
					rethrow_last(rc);
				bool dup = false;
				for (const Cand &x : cands)
					dup = dup || plan_mode(x.r) == plan_mode(r);
				if (dup)
					zg_resize_free(r);
				else
					cands.push_back({ r, 0.0f });
			}
			auto free_cands = [&](zg_resize *keep) {
				for (Cand &x : cands)
					if (x.r != keep)
						zg_resize_free(x.r);
			};
			if (cands.size() < 2) {
				free_cands(nullptr);
				continue;
			}
			try {
				// each candidate runs as a batch of these jobs (persistent launch,
				// side streams), as it would inside this batch
				cudaEvent_t e0 = nullptr, e1 = nullptr;
				cuda_check(cudaEventCreate(&e0), "event");
				cuda_check(cudaEventCreate(&e1), "event");
				const size_t n = std::min(same.size(), kSample);
				std::vector<zg_batch_io> sub_io;
				for (size_t k = 0; k < n; ++k)
					sub_io.push_back(b->io[same[k]]);
				for (Cand &x : cands) {
					std::vector<zg_resize_params> ps(n, x.r->params);
					zg_batch *tb = nullptr;
					if (zg_error_code rc = zg_batch_create(ps.data(), static_cast<unsigned>(n), &tb))
						rethrow_last(rc);
					std::unique_ptr<zg_batch, void (*)(zg_batch *)> hold(tb, zg_batch_free);
					if (zg_error_code rc = zg_batch_set_io(tb, sub_io.data(), stream))
						rethrow_last(rc);
					DeviceBuffer tmp(tb->tmp_size);
					auto run = [&] {
						if (zg_error_code rc = zg_batch_process(tb, tmp.get(), stream))
							rethrow_last(rc);
					};
					run();  // warm-up
					x.ms = 1e30f;
					for (int rep = 0; rep < kReps; ++rep) {
						cuda_check(cudaEventRecord(e0, st), "event");
						run();
						cuda_check(cudaEventRecord(e1, st), "event");
						cuda_check(cudaEventSynchronize(e1), "event");
						float ms = 0.0f;
						cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
						x.ms = std::min(x.ms, ms);
					}
				}
				cudaEventDestroy(e0);
				cudaEventDestroy(e1);
			} catch (...) {
				free_cands(nullptr);
				throw;
			}
			size_t best = 0, current = 0;
			for (size_t c = 0; c < cands.size(); ++c) {
				if (cands[c].ms < cands[best].ms)
					best = c;
				if (plan_mode(cands[c].r) == plan_mode(b->jobs[i]))
					current = c;
			}
			if (plan_mode(cands[best].r) == plan_mode(b->jobs[i]) || cands[best].ms > kMargin * cands[current].ms) {
				free_cands(nullptr);
				continue;
			}
			// the winner's parameters for every job of this kind
			const zg_resize_params chosen = cands[best].r->params;
			free_cands(nullptr);
			for (size_t j : same) {
				zg_resize *r = nullptr;
				if (zg_error_code rc = zg_resize_create(&chosen, &r))
					rethrow_last(rc);
				zg_resize_free(b->jobs[j]);
				b->jobs[j] = r;
				++n_changed;
			}
		}
		if (n_changed) {
			regroup(b);
			upload_io(b, st);
			if (b->graph) {
				cudaGraphExecDestroy(b->graph);
				b->graph = nullptr;
			}
		}
		if (changed)
			*changed = n_changed;
	});
}

zg_error_code zg_batch_get_launch_count(const zg_batch *b, unsigned *out)
{
	return guarded([&] {
		if (!b || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		unsigned n = 0;
		if (b->mixed_now) {
			// one launch for the chained groups and the copies; other groups apart
			n = 1;
			for (const auto &g : b->groups)
				n += g.tma_plan ? 0u : 1u;
		} else {
			n = static_cast<unsigned>(b->groups.size()) + (b->copy_jobs.empty() ? 0u : 1u);
		}
		for (size_t i = 0; i < b->jobs.size(); ++i) {
			if (b->table_index[i] >= 0)
				continue;
			n += static_cast<unsigned>(b->jobs[i]->num_passes);
		}
		*out = n;
	});
}

} // extern "C"
