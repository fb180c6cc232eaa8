// C ABI: a conversion entry point that allocates nothing.
//
// Some callers cannot allocate device memory when they process a frame: a
// video-filter host that hands its plugins only frame buffers from its own
// pool, a real-time loop that must not hit the implicit device-wide
// synchronisation of cudaMalloc/cudaFree, or a process whose allocator is
// owned by another framework. zg_resize_process needs a caller-provided tmp
// buffer for two-pass conversions; this entry point uses a fixed scratch array
// compiled into the library instead.
//
// The array below is a file-scope __device__ object of
// ZG_NO_ALLOC_TMP_BYTES. Every GPU on which this library's module is loaded
// holds it until the process exits: under CUDA's default lazy module loading
// that happens on the library's first kernel launch or symbol lookup on the
// device, under CUDA_MODULE_LOADING=EAGER when the context is created, even
// if this entry point is never called. In host code the array's name is only
// a host-side stand-in, so its device address is obtained with
// cudaGetSymbolAddress, once per device, with that device current, on the
// first call made on that device; later calls read the cached address without
// taking a lock.
#include "capi_common.h"

#include <atomic>
#include <mutex>

namespace {

constexpr size_t kStaticTmpBytes = ZG_NO_ALLOC_TMP_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_tmp[kStaticTmpBytes];

std::mutex g_setup_mutex;
std::atomic<void *> g_static_tmp_addr[kMaxDevices];

// Device address of g_static_tmp on device `dev`, the current device (looked
// up on first use).
void *static_tmp_on_device(int dev)
{
	if (dev < 0 || dev >= kMaxDevices)
		throw zg::Error(zg::kErrUnknown, "device index beyond the library's static scratch table");
	void *addr = g_static_tmp_addr[dev].load(std::memory_order_acquire);
	if (addr)
		return addr;
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	addr = g_static_tmp_addr[dev].load(std::memory_order_relaxed);
	if (!addr) {
		cudaError_t e = cudaGetSymbolAddress(&addr, g_static_tmp);
		if (e != cudaSuccess)
			throw zg::Error(zg::kErrUnknown, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
		if (!addr)
			throw zg::Error(zg::kErrUnknown, "cudaGetSymbolAddress returned a null static scratch address");
		g_static_tmp_addr[dev].store(addr, std::memory_order_release);
	}
	return addr;
}

} // namespace

extern "C" {

zg_error_code zg_resize_process_no_alloc(const zg_resize *r, const void *src, ptrdiff_t src_stride, void *dst,
                                         ptrdiff_t dst_stride, zg_stream stream)
{
	size_t need = 0;
	zg_error_code rc = zg_resize_get_tmp_size(r, &need);
	if (rc != ZG_ERROR_SUCCESS)
		return rc;
	void *tmp = nullptr;
	rc = zg::guarded([&] {
		if (need > kStaticTmpBytes)
			throw zg::Error(zg::kErrOutOfMemory,
			                "conversion needs " + std::to_string(need) + " bytes of scratch; the static scratch of "
			                "zg_resize_process_no_alloc holds " + std::to_string(kStaticTmpBytes) +
			                " bytes (use zg_resize_process with a caller-allocated tmp)");
		if (need) {
			// the plan's device first: a call on another device is a caller
			// error and must not look the array up (or load the module) there
			const int dev = zg::current_device();
			if (!r || dev != r->device)
				throw zg::Error(zg::kErrLogic, "object used on a different device than the one it was created on");
			tmp = static_tmp_on_device(dev);
		}
	});
	if (rc != ZG_ERROR_SUCCESS)
		return rc;
	return zg_resize_process(r, src, src_stride, dst, dst_stride, tmp, stream);
}

} // extern "C"
