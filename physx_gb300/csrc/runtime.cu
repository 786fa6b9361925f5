// Device discovery and small runtime helpers exported through the C ABI.
#include "common.cuh"
#include <cuda_profiler_api.h>
#include <nvtx3/nvToolsExt.h>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>
#include <unistd.h>

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

// ---- host worker pool ----
namespace
{
// Workers sleep on a condition variable; a job hands out chunks through an
// atomic counter that the caller drains too.  The pool is never destroyed (its
// threads end with the process); a child process made by fork() gets a new one.
struct HostPool
{
	std::mutex lock;     // guards the job fields below
	std::mutex runLock;  // one job at a time
	std::condition_variable wake, idle;
	std::vector<std::thread> workers;
	const std::function<void(uint32_t, uint32_t)>* job = nullptr;
	std::atomic<uint32_t> next{0};
	uint32_t total = 0, chunk = 0, busy = 0;
	uint64_t generation = 0;

	explicit HostPool(uint32_t nbWorkers)
	{
		for(uint32_t t = 0; t < nbWorkers; t++) workers.emplace_back([this] { loop(); });
	}
	void drain(const std::function<void(uint32_t, uint32_t)>& fn, uint32_t n, uint32_t c)
	{
		for(;;)
		{
			const uint32_t b = next.fetch_add(c);
			if(b >= n) return;
			fn(b, n - b < c ? n : b + c);
		}
	}
	void loop()
	{
		uint64_t seen = 0;
		for(;;)
		{
			const std::function<void(uint32_t, uint32_t)>* fn;
			uint32_t n, c;
			{
				std::unique_lock<std::mutex> l(lock);
				wake.wait(l, [&] { return generation != seen; });
				seen = generation;
				fn = job;
				n = total;
				c = chunk;
			}
			drain(*fn, n, c);
			std::lock_guard<std::mutex> g(lock);
			if(--busy == 0) idle.notify_one();
		}
	}
	void run(uint32_t n, uint32_t c, const std::function<void(uint32_t, uint32_t)>& fn)
	{
		std::lock_guard<std::mutex> serial(runLock);
		{
			std::lock_guard<std::mutex> g(lock);
			job = &fn;
			total = n;
			chunk = c;
			next.store(0);
			busy = uint32_t(workers.size());
			generation++;
		}
		wake.notify_all();
		drain(fn, n, c);
		std::unique_lock<std::mutex> l(lock);
		idle.wait(l, [&] { return busy == 0; });
	}
};
std::mutex gPoolLock;
HostPool* gPool = nullptr;
pid_t gPoolPid = 0;
} // namespace

void hostParallelFor(uint32_t n, uint32_t chunk, const std::function<void(uint32_t, uint32_t)>& fn)
{
	if(chunk == 0) chunk = 1;
	if(n <= chunk)
	{
		if(n) fn(0, n);
		return;
	}
	HostPool* pool;
	{
		std::lock_guard<std::mutex> g(gPoolLock);
		if(!gPool || gPoolPid != getpid())
		{
			const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
			gPool = new HostPool(std::min(7u, hw - 1));   // a pool left by the parent process is abandoned
			gPoolPid = getpid();
		}
		pool = gPool;
	}
	if(pool->workers.empty()) fn(0, n);
	else pool->run(n, chunk, fn);
}
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
