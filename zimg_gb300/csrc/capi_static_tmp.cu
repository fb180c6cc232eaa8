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
// ZG_NO_ALLOC_TMP_BYTES. Every GPU that loads this library's module holds it
// from the first call on that device until the process exits. In host code
// its name is only a host-side stand-in, so its device address is obtained
// with cudaGetSymbolAddress, once per device, with that device current, on the
// first call made on that device.
#include "capi_common.h"

#include <mutex>

namespace {

constexpr size_t kStaticTmpBytes = ZG_NO_ALLOC_TMP_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_tmp[kStaticTmpBytes];

std::mutex g_setup_mutex;
void *g_static_tmp_addr[kMaxDevices] = {};

// Device address of g_static_tmp on the current device (set up on first use).
void *static_tmp_on_current_device()
{
	const int dev = zg::current_device();
	if (dev < 0 || dev >= kMaxDevices)
		throw zg::Error(zg::kErrUnknown, "device index beyond the library's static scratch table");
	std::lock_guard<std::mutex> lock(g_setup_mutex);
	if (!g_static_tmp_addr[dev]) {
		void *addr = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&addr, g_static_tmp);
		if (e != cudaSuccess)
			throw zg::Error(zg::kErrUnknown, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
		if (!addr)
			throw zg::Error(zg::kErrUnknown, "cudaGetSymbolAddress returned a null static scratch address");
		g_static_tmp_addr[dev] = addr;
	}
	return g_static_tmp_addr[dev];
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
		if (need)
			tmp = static_tmp_on_current_device();
	});
	if (rc != ZG_ERROR_SUCCESS)
		return rc;
	return zg_resize_process(r, src, src_stride, dst, dst_stride, tmp, stream);
}

} // extern "C"
