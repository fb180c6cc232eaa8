/*
 * Minimal stand-in for the graphengine filter interface, written from the way
 * zimg's resize code uses it (src/zimg/graph/filter_base.h:14-23,
 * src/zimg/resize/resize_impl.cpp:21-28,130-160, src/zimg/api/zimg.h:387-396).
 *
 * The graphengine submodule is not part of the reference checkout, so the
 * reference's resize sources cannot be compiled without a header that supplies
 * these types. Only the members that the resize filters read or write are
 * provided. This file is test infrastructure for the oracle build only.
 */
#pragma once

#ifndef ORACLE_GRAPHENGINE_FILTER_H_
#define ORACLE_GRAPHENGINE_FILTER_H_

#include <cstddef>
#include <utility>

namespace graphengine {

struct PlaneDescriptor {
	unsigned width;
	unsigned height;
	unsigned bytes_per_sample;
};

/* Line i of a buffer lives at ptr + (i & mask) * stride (zimg.h:394-396). */
struct BufferDescriptor {
	void *ptr;
	std::ptrdiff_t stride;
	unsigned mask;

	template <class T = void>
	T *get_line(unsigned i) const
	{
		return reinterpret_cast<T *>(static_cast<unsigned char *>(ptr) + static_cast<std::ptrdiff_t>(i & mask) * stride);
	}
};

struct FilterFlags {
	bool stateful;
	bool in_place;
	bool entire_row;
	bool entire_col;
};

struct FilterDescriptor {
	PlaneDescriptor format;
	unsigned num_deps;
	unsigned num_planes;
	unsigned step;
	unsigned alignment_mask;
	std::size_t context_size;
	std::size_t scratchpad_size;
	FilterFlags flags;
};

class Filter {
public:
	typedef std::pair<unsigned, unsigned> pair_unsigned;

	static constexpr int VERSION = 1;

	virtual ~Filter() = default;

	virtual int version() const noexcept = 0;

	virtual const FilterDescriptor &descriptor() const noexcept = 0;

	virtual pair_unsigned get_row_deps(unsigned i) const noexcept = 0;

	virtual pair_unsigned get_col_deps(unsigned left, unsigned right) const noexcept = 0;

	virtual void init_context(void *context) const noexcept = 0;

	virtual void process(const BufferDescriptor *in, const BufferDescriptor *out,
	                     unsigned i, unsigned left, unsigned right, void *context, void *tmp) const noexcept = 0;
};

} // namespace graphengine

#endif // ORACLE_GRAPHENGINE_FILTER_H_
