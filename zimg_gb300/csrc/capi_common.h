// Shared host-side pieces of the C ABI: error capture, device buffers and the
// device copy of a pass's tap tables.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "filter_plan.h"
#include "fused.h"
#include "kernels.h"
#include "zimg_gb300.h"

namespace zg {

// Record the last error on this thread (zimg.cpp:33-34,61-105).
void set_last_error(int code, const std::string &msg);

// Run f; map exceptions to zg_error_code and the thread-local message.
template <class F>
zg_error_code guarded(F &&f) noexcept
{
	try {
		f();
		return ZG_ERROR_SUCCESS;
	} catch (const Error &e) {
		set_last_error(e.code, e.what());
		return static_cast<zg_error_code>(e.code);
	} catch (const std::bad_alloc &) {
		set_last_error(ZG_ERROR_OUT_OF_MEMORY, "out of memory");
		return ZG_ERROR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		set_last_error(ZG_ERROR_UNKNOWN, e.what());
		return ZG_ERROR_UNKNOWN;
	} catch (...) {
		set_last_error(ZG_ERROR_UNKNOWN, "unknown error");
		return ZG_ERROR_UNKNOWN;
	}
}

inline void cuda_check(cudaError_t e, const char *what)
{
	if (e == cudaErrorMemoryAllocation)
		throw Error(kErrOutOfMemory, std::string(what) + ": " + cudaGetErrorString(e));
	if (e != cudaSuccess)
		throw Error(kErrUnknown, std::string(what) + ": " + cudaGetErrorString(e));
}

// A plane copy of `rows` lines of `row_bytes` on `st`; strides may be
// negative (zimg_image_buffer allows them, zimg.h:387-433). Both negative:
// the same rows walked from the last one with positive pitches; one negative:
// line by line.
inline void copy_plane(void *dst, ptrdiff_t ds, const void *src, ptrdiff_t ss, size_t row_bytes, unsigned rows,
                       cudaStream_t st)
{
	if (!rows || !row_bytes)
		return;
	if (ds >= 0 && ss >= 0) {
		cuda_check(cudaMemcpy2DAsync(dst, static_cast<size_t>(ds), src, static_cast<size_t>(ss), row_bytes, rows,
		                             cudaMemcpyDeviceToDevice, st), "plane copy");
	} else if (ds < 0 && ss < 0) {
		char *d = static_cast<char *>(dst) + static_cast<ptrdiff_t>(rows - 1) * ds;
		const char *s = static_cast<const char *>(src) + static_cast<ptrdiff_t>(rows - 1) * ss;
		cuda_check(cudaMemcpy2DAsync(d, static_cast<size_t>(-ds), s, static_cast<size_t>(-ss), row_bytes, rows,
		                             cudaMemcpyDeviceToDevice, st), "plane copy");
	} else {
		for (unsigned i = 0; i < rows; ++i)
			cuda_check(cudaMemcpyAsync(static_cast<char *>(dst) + static_cast<ptrdiff_t>(i) * ds,
			                           static_cast<const char *>(src) + static_cast<ptrdiff_t>(i) * ss, row_bytes,
			                           cudaMemcpyDeviceToDevice, st),
			           "plane copy");
	}
}

inline ptrdiff_t abs_stride(ptrdiff_t s)
{
	return s < 0 ? -s : s;
}

// Owned device allocation made at plan-creation time.
class DeviceBuffer {
public:
	DeviceBuffer() = default;
	explicit DeviceBuffer(size_t bytes) { reset(bytes); }
	~DeviceBuffer() { release(); }
	DeviceBuffer(const DeviceBuffer &) = delete;
	DeviceBuffer &operator=(const DeviceBuffer &) = delete;

	void reset(size_t bytes)
	{
		release();
		if (bytes)
			cuda_check(cudaMalloc(&ptr_, bytes), "cudaMalloc");
		size_ = bytes;
	}
	void release()
	{
		if (ptr_)
			cudaFree(ptr_);
		ptr_ = nullptr;
		size_ = 0;
	}
	void *get() const { return ptr_; }
	size_t size() const { return size_; }

private:
	void *ptr_ = nullptr;
	size_t size_ = 0;
};

// Device copy of one FilterTable plus its geometry.
struct DevicePass {
	FilterTable table;        // host copy (kept for introspection)
	DeviceBuffer storage;     // left | f32 | i16 | bias
	PassTables tables{};
	bool horizontal = false;
	Sample sample = Sample::F32;
	int32_t pixel_max = 0;
	unsigned src_w = 0, src_h = 0, dst_w = 0, dst_h = 0;
	// FP32 only: band fragments for the tensor-core kernel (set_tensor)
	DeviceBuffer wide_storage;
	WideTables wide{};

	void upload();
	void set_tensor();
};

// FP32 passes with at least this many taps run on the tensor cores under
// ZG_ENGINE_AUTO when they are not fused.
constexpr unsigned kWideTaps = 32;

struct PassSpec {
	unsigned src_w, src_h;
	Sample sample;
	unsigned depth;
	bool horizontal;
	unsigned dst_dim;
	int filter;
	double a, b;
	double shift, subwidth;
};

std::unique_ptr<DevicePass> make_device_pass(const PassSpec &s);

inline double default_extent(double v, unsigned dim)
{
	return (std::isnan(v) || v <= 0.0) ? static_cast<double>(dim) : v;
}

Sample sample_of(int pixel_type);
unsigned bytes_of(Sample s);
int current_device();

} // namespace zg

// A conversion: zero, one or two passes, optionally fused into one kernel.
struct zg_resize {
	int device;
	zg_resize_params params;
	int num_passes = 0;
	bool first_horizontal = false;
	bool fused = false;
	bool tensor_passes = false;  // separate passes, at least one on the tensor cores
	std::unique_ptr<zg::DevicePass> pass[2];
	ptrdiff_t tmp_stride = 0;
	size_t tmp_size = 0;
	zg::Sample sample = zg::Sample::F32;
	zg::FusedPlan fplan;
	zg::DeviceBuffer fblob;
	zg::SmemLayout flayout{};
	int fgrid = 0;
	// chained plans: the TMA-pipelined kernel's layout, used when the source
	// plane admits a tensor map
	bool tma = false;
	zg::SmemLayout tlayout{};
	int tgrid = 0;
};
