// Device discovery and small runtime helpers exported through the C ABI.
#include "common.cuh"
#include <cuda_profiler_api.h>

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
