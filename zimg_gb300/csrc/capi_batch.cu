// C ABI: batches of conversions over planes of uneven sizes.
#include "capi_common.h"

#include <algorithm>

using namespace zg;

struct zg_batch {
	int device;
	std::vector<zg_resize *> jobs;
	std::vector<size_t> tmp_offset;
	size_t tmp_size = 0;
	std::vector<zg_batch_io> io;
	cudaGraphExec_t graph = nullptr;
	cudaStream_t graph_stream = nullptr;
	void *graph_tmp = nullptr;

	~zg_batch()
	{
		if (graph)
			cudaGraphExecDestroy(graph);
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

void batch_launch(const zg_batch *b, void *tmp, cudaStream_t st)
{
	if (b->io.size() != b->jobs.size())
		throw Error(kErrLogic, "zg_batch_set_io was not called");
	for (size_t i = 0; i < b->jobs.size(); ++i) {
		const zg_batch_io &io = b->io[i];
		void *t = b->tmp_size ? static_cast<char *>(tmp) + b->tmp_offset[i] : nullptr;
		zg_error_code rc = zg_resize_process(b->jobs[i], io.src, io.src_stride, io.dst, io.dst_stride, t,
		                                     reinterpret_cast<zg_stream>(st));
		if (rc != ZG_ERROR_SUCCESS)
			rethrow_last(rc);
	}
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
			size_t t = 0;
			zg_resize_get_tmp_size(r, &t);
			b->tmp_offset.push_back(b->tmp_size);
			b->tmp_size += (t + 255) & ~static_cast<size_t>(255);
		}
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
		(void)stream;
		b->io.assign(io, io + b->jobs.size());
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

zg_error_code zg_batch_get_launch_count(const zg_batch *b, unsigned *out)
{
	return guarded([&] {
		if (!b || !out)
			throw Error(kErrIllegalArgument, "null pointer");
		unsigned n = 0;
		for (auto *j : b->jobs) {
			int passes = 0, first = 0, fused = 0;
			zg_resize_get_info(j, &passes, &first, &fused);
			n += fused ? 1 : static_cast<unsigned>(passes);
		}
		*out = n;
	});
}

} // extern "C"
