// Device discovery and small runtime helpers exported through the C ABI.
#include "common.cuh"
#include <cuda_profiler_api.h>
#include <nvtx3/nvToolsExt.h>
#include <atomic>

GBPX_API int gbpx_device_count(int* out)
{
	if(!out) return GBPX_ERR_INVALID;
	int n = 0;
	if(cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); n = 0; }
	*out = n;
	return GBPX_OK;
}

// name (up to 256 bytes), SM count, compute capability major*10+minor.
GBPX_API int gbpx_device_info(int device, char* name, int nameBytes, int* smCount, int* cc)
{
	cudaDeviceProp p;
	GBPX_CUDA_TRY(cudaGetDeviceProperties(&p, device));
	if(name && nameBytes > 0) { strncpy(name, p.name, size_t(nameBytes) - 1); name[nameBytes - 1] = 0; }
	if(smCount) *smCount = p.multiProcessorCount;
	if(cc) *cc = p.major * 10 + p.minor;
	return GBPX_OK;
}

GBPX_API int gbpx_device_synchronize(void)
{
	GBPX_CUDA_TRY(cudaDeviceSynchronize());
	return GBPX_OK;
}

GBPX_API int gbpx_set_device(int device)
{
	GBPX_CUDA_TRY(cudaSetDevice(device));
	return GBPX_OK;
}

// Profiler range (cudaProfilerStart/Stop): a profiler started with its capture
// off records only the kernels launched inside the range.
GBPX_API int gbpx_profiler_start(void)
{
	GBPX_CUDA_TRY(cudaProfilerStart());
	return GBPX_OK;
}

GBPX_API int gbpx_profiler_stop(void)
{
	GBPX_CUDA_TRY(cudaDeviceSynchronize());
	GBPX_CUDA_TRY(cudaProfilerStop());
	return GBPX_OK;
}

// ---- profiler zones ----
namespace gbpx
{
namespace
{
struct ZoneHooks
{
	ZoneStartFn start;
	ZoneEndFn end;
	void* user;
};
std::atomic<const ZoneHooks*> gHooks{nullptr};
ZoneHooks gHookSlots[2];
std::atomic<uint32_t> gHookSlot{0};
} // namespace

void zoneCallbacks(ZoneStartFn* start, ZoneEndFn* end, void** user)
{
	const ZoneHooks* h = gHooks.load(std::memory_order_acquire);
	if(h) { *start = h->start; *end = h->end; *user = h->user; }
	else { *start = nullptr; *end = nullptr; *user = nullptr; }
}

void nvtxPush(const char* name) { nvtxRangePushA(name); }
void nvtxPop() { nvtxRangePop(); }
} // namespace gbpx

// Installs (or, with null functions, removes) the callbacks every profiler
// zone calls: zoneStart(name, detached, contextId, user) returns a value that
// zoneEnd(value, name, detached, contextId, user) gets back (the reference's
// PxProfilerCallback protocol, physx/include/foundation/PxProfiler.h:58-69).
// Set it while no library call is running.
GBPX_API int gbpx_set_profiler_callback(gbpx::ZoneStartFn zoneStart, gbpx::ZoneEndFn zoneEnd, void* user)
{
	if((zoneStart == nullptr) != (zoneEnd == nullptr)) return GBPX_ERR_INVALID;
	if(!zoneStart)
	{
		gbpx::gHooks.store(nullptr, std::memory_order_release);
		return GBPX_OK;
	}
	const uint32_t slot = gbpx::gHookSlot.fetch_add(1) & 1u;
	gbpx::gHookSlots[slot] = gbpx::ZoneHooks{zoneStart, zoneEnd, user};
	gbpx::gHooks.store(&gbpx::gHookSlots[slot], std::memory_order_release);
	return GBPX_OK;
}
