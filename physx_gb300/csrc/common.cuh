// Shared device/host helpers for the GB300 rigid-body step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <functional>
#include <utility>

#define GBPX_API extern "C" __attribute__((visibility("default")))

// Status codes returned through the C ABI (include/gbpx.h mirrors them).
enum GbpxStatus
{
	GBPX_OK = 0,
	GBPX_ERR_INVALID = -1,      // bad argument (null pointer, size out of range)
	GBPX_ERR_CUDA = -2,         // a CUDA runtime call failed
	GBPX_ERR_CAPACITY = -3,     // a device buffer overflowed; retried once then reported
	GBPX_ERR_NOMEM = -4,        // device allocation failed
	GBPX_ERR_STATE = -5,        // call sequence violated (e.g. fetch without update)
	GBPX_ERR_BUDGET = -6,       // memory budget exceeded (serving admission)
	GBPX_ERR_TIMEOUT = -7,      // a bounded device wait gave up
};

#define GBPX_CUDA_TRY(expr)                                                                   \
	do {                                                                                      \
		cudaError_t _e = (expr);                                                              \
		if(_e != cudaSuccess) {                                                               \
			fprintf(stderr, "[gbpx] CUDA error %s at %s:%d: %s\n", cudaGetErrorName(_e),     \
			        __FILE__, __LINE__, cudaGetErrorString(_e));                              \
			return GBPX_ERR_CUDA;                                                             \
		}                                                                                     \
	} while(0)

namespace gbpx
{
static inline uint32_t divUp(uint64_t a, uint32_t b) { return uint32_t((a + b - 1) / b); }

// Profiler zones, as the reference marks its stages with PX_PROFILE_ZONE
// (physx/include/common/PxProfileZone.h): each zone is an NVTX range (seen by
// Nsight tools) and, when the user installed callbacks with
// gbpx_set_profiler_callback, a zoneStart / zoneEnd pair on them.  Zones are
// host-side: they bracket the launches and copies of a stage.
typedef void* (*ZoneStartFn)(const char* name, int detached, uint64_t contextId, void* user);
typedef void (*ZoneEndFn)(void* data, const char* name, int detached, uint64_t contextId, void* user);
void zoneCallbacks(ZoneStartFn* start, ZoneEndFn* end, void** user);
void nvtxPush(const char* name);
void nvtxPop();
struct Zone
{
	const char* name;
	uint64_t context;
	void* data = nullptr;
	ZoneStartFn start = nullptr;
	ZoneEndFn end = nullptr;
	void* user = nullptr;
	Zone(const char* n, uint64_t ctx = 0) : name(n), context(ctx)
	{
		nvtxPush(n);
		zoneCallbacks(&start, &end, &user);
		if(start) data = start(n, 0, ctx, user);
	}
	~Zone()
	{
		if(end) end(data, name, 0, context, user);
		nvtxPop();
	}
	Zone(const Zone&) = delete;
	Zone& operator=(const Zone&) = delete;
};

// Host-side parallel loop over [0, n) in chunks of `chunk` items, run by a
// process-wide pool of worker threads (created on first use, at most 7 workers
// plus the caller) so that large host gathers do not pay a thread start each
// call.  fn(begin, end) must be safe to run concurrently on disjoint ranges.
// Calls from several threads are serialised.  Falls back to the caller alone
// when n <= chunk.
void hostParallelFor(uint32_t n, uint32_t chunk, const std::function<void(uint32_t, uint32_t)>& fn);

// Device buffer that only grows; contents are not preserved across growth unless asked.
template <typename T>
struct DevBuf
{
	T* ptr = nullptr;
	size_t cap = 0;
	int reserve(size_t n, cudaStream_t s = 0, bool keep = false, size_t keepCount = 0)
	{
		if(n <= cap) return GBPX_OK;
		// first allocation exact (large resident pools); later growth doubles
		size_t nc = cap ? cap : n;
		while(nc < n) nc *= 2;
		T* np = nullptr;
		if(cudaMalloc(&np, nc * sizeof(T)) != cudaSuccess) return GBPX_ERR_NOMEM;
		if(keep && ptr && keepCount)
			if(cudaMemcpyAsync(np, ptr, keepCount * sizeof(T), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return GBPX_ERR_CUDA;
		if(ptr) { cudaStreamSynchronize(s); cudaFree(ptr); }
		ptr = np;
		cap = nc;
		return GBPX_OK;
	}
	void release() { if(ptr) cudaFree(ptr); ptr = nullptr; cap = 0; }
};

template <typename T>
struct HostBuf
{
	T* ptr = nullptr;
	size_t cap = 0;
	int reserve(size_t n, bool keep = false)
	{
		if(n <= cap) return GBPX_OK;
		// first allocation exact (large resident pools); later growth doubles
		size_t nc = cap ? cap : n;
		while(nc < n) nc *= 2;
		T* np = nullptr;
		if(cudaMallocHost(&np, nc * sizeof(T)) != cudaSuccess) return GBPX_ERR_NOMEM;
		if(keep && ptr) memcpy(np, ptr, cap * sizeof(T));
		if(ptr) cudaFreeHost(ptr);
		ptr = np;
		cap = nc;
		return GBPX_OK;
	}
	void release() { if(ptr) cudaFreeHost(ptr); ptr = nullptr; cap = 0; }
};

// IEEE-754 float bits -> order-preserving unsigned key (negatives reversed,
// positives shifted above them).  -0.0 maps just below +0.0.
__host__ __device__ __forceinline__ uint32_t encodeFloatBits(uint32_t ir)
{
	return (ir & 0x80000000u) ? ~ir : (ir | 0x80000000u);
}

__device__ __forceinline__ uint32_t laneMaskLt()
{
	uint32_t m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// Programmatic dependent launch: a kernel launched with launchDependent() may
// start while the previous kernel in the stream is finishing; it must call
// gridDependencyWait() before touching anything that kernel writes (the wait
// returns once the previous grid has completed and its writes are visible),
// and may call gridLaunchDependents() to let the next such launch begin.
__device__ __forceinline__ void gridDependencyWait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void gridLaunchDependents() { asm volatile("griddepcontrol.launch_dependents;\n" :::); }
template <typename... Params, typename... Args>
inline cudaError_t launchDependent(void (*kernel)(Params...), uint32_t grid, uint32_t block, cudaStream_t stream, Args&&... args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(block);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = stream;
	cudaLaunchAttribute attr;
	attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr.val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = &attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Asynchronous 16-byte global -> shared copy (cp.async; complete in the issuing
// thread after cpAsyncWaitAll).  Both addresses must be 16-byte aligned.
__device__ __forceinline__ void cpAsync16(void* smem, const void* gmem)
{
	const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
} // namespace gbpx
