/*
 * C++ adapter: a zimg_gb300 resize pass behind the interface of zimg's graph
 * filters, so host code that builds a filter graph out of
 * graphengine::Filter objects can put it where ResizeImplH / ResizeImplV
 * stood (src/zimg/resize/resize_impl.h:18-43, built by ResizeImplBuilder,
 * resize_impl.cpp:245-267; interface src/zimg/graph/filter_base.h:14-23).
 *
 * The filter is whole-plane: it asks for every input line and column, and
 * process() runs the pass over the whole plane on the GPU when it is called
 * for output line 0, doing nothing for the other lines. So the graph must hand
 * it device planes held whole (mask == ZG_BUFFER_MAX), as zimg does for
 * filters whose descriptor sets entire_row / entire_col; its left / right
 * range, context and tmp are not used.
 *
 * The class is a template over the host's graphengine types, so this header
 * does not depend on graphengine:
 *
 *   using GpuResizePass = zg::GraphengineResizePass<graphengine::Filter,
 *                                                   graphengine::BufferDescriptor,
 *                                                   graphengine::FilterDescriptor>;
 *   zg_pass_params p = ...;            // what ResizeImplBuilder takes
 *   auto f = std::make_unique<GpuResizePass>(p, stream);
 *
 * FilterBase must provide pair_unsigned, VERSION and the virtual functions
 * below; BufferDescriptor the members ptr and stride; FilterDescriptor the
 * members format.{width,height,bytes_per_sample}, num_deps, num_planes, step,
 * alignment_mask, context_size, scratchpad_size and flags.{stateful, in_place,
 * entire_row, entire_col}.
 */
#ifndef ZIMG_GB300_FILTER_HPP_
#define ZIMG_GB300_FILTER_HPP_

#include <stdexcept>
#include <string>

#include "zimg_gb300.h"

namespace zg {

/* A failed zimg_gb300 call: zimg's error code and the thread's message. */
class Exception : public std::runtime_error {
public:
	zg_error_code code;
	Exception(zg_error_code c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

inline void check(zg_error_code rc)
{
	if (rc != ZG_ERROR_SUCCESS) {
		char msg[512];
		zg_get_last_error(msg, sizeof(msg));
		throw Exception(rc, msg);
	}
}

template <class FilterBase, class BufferDescriptor, class FilterDescriptor>
class GraphengineResizePass : public FilterBase {
public:
	using pair_unsigned = typename FilterBase::pair_unsigned;

	/* Throws zg::Exception with zimg's error code when the pass cannot be built. */
	explicit GraphengineResizePass(const zg_pass_params &p, zg_stream stream = nullptr)
		: m_src_w(p.src_width), m_src_h(p.src_height), m_stream(stream)
	{
		check(zg_resize_pass_create(&p, &m_pass));
		unsigned w = 0, h = 0;
		check(zg_resize_pass_get_output(m_pass, &w, &h));
		m_desc.format.width = w;
		m_desc.format.height = h;
		m_desc.format.bytes_per_sample = p.pixel_type == ZG_PIXEL_WORD ? 2 : 4;
		m_desc.num_deps = 1;
		m_desc.num_planes = 1;
		m_desc.step = h;
		m_desc.alignment_mask = 0;
		m_desc.context_size = 0;
		m_desc.scratchpad_size = 0;
		m_desc.flags.stateful = false;
		m_desc.flags.in_place = false;
		m_desc.flags.entire_row = true;
		m_desc.flags.entire_col = true;
	}

	~GraphengineResizePass() override { zg_resize_pass_free(m_pass); }

	GraphengineResizePass(const GraphengineResizePass &) = delete;
	GraphengineResizePass &operator=(const GraphengineResizePass &) = delete;

	int version() const noexcept override { return FilterBase::VERSION; }

	const FilterDescriptor &descriptor() const noexcept override { return m_desc; }

	pair_unsigned get_row_deps(unsigned) const noexcept override { return { 0, m_src_h }; }

	pair_unsigned get_col_deps(unsigned, unsigned) const noexcept override { return { 0, m_src_w }; }

	void init_context(void *) const noexcept override {}

	/* Line 0: the whole pass, enqueued on the stream given at construction.
	 * process() cannot throw (graphengine's interface is noexcept): a failure
	 * is left in zg_get_last_error() and in status(). */
	void process(const BufferDescriptor *in, const BufferDescriptor *out, unsigned i, unsigned, unsigned, void *,
	             void *) const noexcept override
	{
		if (i != 0)
			return;
		m_status = zg_resize_pass_process(m_pass, in->ptr, in->stride, out->ptr, out->stride, m_stream);
	}

	/* Result of the last whole-plane process() call. */
	zg_error_code status() const noexcept { return m_status; }

private:
	zg_resize_pass *m_pass = nullptr;
	FilterDescriptor m_desc{};
	unsigned m_src_w, m_src_h;
	zg_stream m_stream;
	mutable zg_error_code m_status = ZG_ERROR_SUCCESS;
};

} // namespace zg

#endif /* ZIMG_GB300_FILTER_HPP_ */
