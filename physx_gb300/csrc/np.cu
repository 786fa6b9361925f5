// Narrowphase for the GB300 rigid-body step: immediate::PxGenerateContacts
// (physx/include/PxImmediateMode.h:267, physx/source/immediatemode/src/NpImmediateMode.cpp:732)
// over a batch of sphere / plane / capsule / box / convex-core pairs, with
// fresh caches or with each pair's persistent contact manifold carried between
// calls (convex-core pairs keep none).
//
// GB300 layout: the batch is bucketed by (type0, type1) with a counting pass
// (16 bins for the sphere/plane/capsule/box kinds, then the pairs with a convex
// core by shape and core types, which come last) so every warp runs a single generator (no
// divergence between pair types); the convex-core pairs run in their own
// kernel, whose GJK/EPA working set does not weigh on the others' registers.
// Each lane runs one pair and writes its <= 4 contacts as float4 pairs
// (normal|separation, point|0) into a fixed 4-slot record, so no compaction is
// needed and the host reads counts + records in one copy.
#include "common.cuh"
#include "contacts.cuh"
#include "convex_core.cuh"
#include <atomic>
#include <mutex>

namespace gbpx
{
namespace np
{
struct PairRef   // one pair of the caller's batch (AoS arrays of the C ABI)
{
	const int* type0; const float* geom0; const int* type1; const float* geom1; const float* pose0; const float* pose1;
};

__device__ __forceinline__ Tr loadPose7(const float* p)
{
	Tr t;
	t.q.x = p[0]; t.q.y = p[1]; t.q.z = p[2]; t.q.w = p[3];
	t.p = v3(p[4], p[5], p[6]);
	return t;
}

// 16 bins for the primitive kinds, then the convex-core pairs: 24 bins for a
// primitive (sphere / plane / capsule / box) against each of the 6 core types,
// 36 for the ordered pairs of core types
constexpr uint32_t NP_BINS = 16 + 24 + 36;

// a shape type's PxGeometryType (the low byte; a convex core carries its core type above it)
__device__ __forceinline__ int geomType(int t) { return t & 0xff; }
__device__ __forceinline__ uint32_t coreType(int t) { const uint32_t c = uint32_t(t) >> 8; return c < 6u ? c : 5u; }
__device__ __forceinline__ bool convexCorePair(int t0, int t1) { return geomType(t0) == 4 || geomType(t1) == 4; }

// the pair's bucket: the convex-core pairs come after the primitive kinds, split
// by core types, so that a warp runs one core type's support and face code
__device__ __forceinline__ uint32_t pairKey(int t0, int t1)
{
	const int g0 = geomType(t0), g1 = geomType(t1);
	if(g0 == 4 && g1 == 4)
	{
		const uint32_t c0 = coreType(t0), c1 = coreType(t1);
		return 40u + (c0 < c1 ? c0 * 6u + c1 : c1 * 6u + c0);
	}
	if(g0 == 4) return 16u + uint32_t(g1 & 3) * 6u + coreType(t0);
	if(g1 == 4) return 16u + uint32_t(g0 & 3) * 6u + coreType(t1);
	const int a = g0 < g1 ? g0 : g1, b = g0 < g1 ? g1 : g0;
	return uint32_t(((a & 3) << 2) | (b & 3));
}

__global__ void bucketCountKernel(PairRef pr, uint32_t n, uint32_t* __restrict__ hist)
{
	__shared__ uint32_t h[NP_BINS];
	if(threadIdx.x < NP_BINS) h[threadIdx.x] = 0;
	__syncthreads();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) atomicAdd(&h[pairKey(pr.type0[i], pr.type1[i])], 1u);
	__syncthreads();
	if(threadIdx.x < NP_BINS && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

__global__ void bucketOffsetsKernel(uint32_t* __restrict__ hist)
{
	if(threadIdx.x == 0)
	{
		uint32_t run = 0;
		for(uint32_t k = 0; k < NP_BINS; k++) { const uint32_t c = hist[k]; hist[k] = run; hist[NP_BINS + k] = run; run += c; }
	}
}

__global__ void bucketScatterKernel(PairRef pr, uint32_t n, uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const uint32_t slot = atomicAdd(&cursor[pairKey(pr.type0[i], pr.type1[i])], 1u);
	perm[slot] = i;
}

// One lane per pair (in bucket order) of slots [0, n) of perm; convex-core pairs
// are left to generateConvexCoreKernel.  out: n x 4 contacts x 2 float4.
// manifolds: per pair, the persistent manifold read and updated (null: fresh caches).
__global__ void __launch_bounds__(128) generateKernel(PairRef pr, const uint32_t* __restrict__ perm, uint32_t n, float contactDistance,
                                                      float toleranceLength, float4* __restrict__ out, uint32_t* __restrict__ counts,
                                                      ManifoldRecord* __restrict__ manifolds)
{
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= n) return;
	const uint32_t i = perm[k];
	int ta = pr.type0[i], tb = pr.type1[i];
	if(convexCorePair(ta, tb)) return;
	float ga[4], gb[4];
#pragma unroll
	for(int c = 0; c < 4; c++) { ga[c] = pr.geom0[4 * size_t(i) + c]; gb[c] = pr.geom1[4 * size_t(i) + c]; }
	Tr pa = loadPose7(pr.pose0 + 7 * size_t(i)), pb = loadPose7(pr.pose1 + 7 * size_t(i));
	const bool swap = ta > tb;
	if(swap)
	{
		const int t = ta; ta = tb; tb = t;
		for(int c = 0; c < 4; c++) { const float x = ga[c]; ga[c] = gb[c]; gb[c] = x; }
		const Tr t2 = pa; pa = pb; pb = t2;
	}
	Buffer buf;
	Manifold m;
	const bool cached = manifolds && cachedKind(ta, tb);
	if(cached) loadManifold(manifolds[i], m);
	generate(ta, ga, tb, gb, pa, pb, contactDistance, toleranceLength, m, buf);
	if(cached) storeManifold(m, manifolds[i]);
	counts[i] = uint32_t(buf.count);
	float4* o = out + size_t(i) * 8;
	for(int c = 0; c < buf.count; c++)
	{
		V3 nn = buf.c[c].n;
		if(swap) nn = neg(nn);
		o[2 * c] = make_float4(nn.x, nn.y, nn.z, buf.c[c].sep);
		o[2 * c + 1] = make_float4(buf.c[c].p.x, buf.c[c].p.y, buf.c[c].p.z, 0.0f);
	}
}
// One lane per convex-core pair among slots [begin, end) of perm (the other
// kinds are skipped): contactPlaneConvexCore / contactConvexCoreConvex with the
// shapes in the reference's table order and the normals negated when swapped.
__global__ void __launch_bounds__(128) generateConvexCoreKernel(PairRef pr, const uint32_t* __restrict__ perm, uint32_t begin, uint32_t end,
                                                                float contactDistance, float4* __restrict__ out, uint32_t* __restrict__ counts)
{
	const uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(k >= end) return;
	const uint32_t i = perm[k];
	int ta = pr.type0[i], tb = pr.type1[i];
	if(!convexCorePair(ta, tb)) return;
	const float* ga = pr.geom0 + 4 * size_t(i);
	const float* gb = pr.geom1 + 4 * size_t(i);
	Tr pa = loadPose7(pr.pose0 + 7 * size_t(i)), pb = loadPose7(pr.pose1 + 7 * size_t(i));
	const bool swap = geomType(ta) > geomType(tb);
	if(swap)
	{
		const int t = ta; ta = tb; tb = t;
		const float* g = ga; ga = gb; gb = g;
		const Tr t2 = pa; pa = pb; pb = t2;
	}
	V3 normal = v3(0.0f, 0.0f, 0.0f), points[cc::MAX_CONTACTS];
	float dists[cc::MAX_CONTACTS];
	const uint32_t c = cc::generatePair(ta, ga, tb, gb, pa, pb, contactDistance, normal, points, dists);
	counts[i] = c;
	if(swap) normal = neg(normal);
	float4* o = out + size_t(i) * 8;
	for(uint32_t j = 0; j < c; j++)
	{
		o[2 * j] = make_float4(normal.x, normal.y, normal.z, dists[j]);
		o[2 * j + 1] = make_float4(points[j].x, points[j].y, points[j].z, 0.0f);
	}
}
} // namespace np

// Per-call device workspace of the immediate-mode narrowphase entry point.
struct NpWorkspace
{
	cudaStream_t stream = 0;
	DevBuf<int> t0, t1;
	DevBuf<float> g0, g1, p0, p1;
	DevBuf<uint32_t> hist, perm, counts;
	DevBuf<float4> out;
	DevBuf<np::ManifoldRecord> manifolds;
	HostBuf<float4> hOut;
	HostBuf<uint32_t> hCounts;
	int init() { GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)); return GBPX_OK; }
};

static NpWorkspace* npWorkspace()
{
	static NpWorkspace* ws = nullptr;
	if(!ws)
	{
		ws = new NpWorkspace;
		if(ws->init()) { delete ws; ws = nullptr; }
	}
	return ws;
}
} // namespace gbpx

using namespace gbpx;

// a shape type this narrowphase generates for: PxGeometryType 0..3, or 4 (convex
// core) with a PxConvexCore::Type 0..5 in bits 8..15
static bool validShapeType(int t)
{
	const uint32_t u = uint32_t(t);
	if(u <= 3u) return true;
	return (u & 0xffu) == 4u && (u >> 8) < uint32_t(cc::CORE_COUNT);
}

// PxGenerateContacts over nbPairs pairs (host arrays, fresh caches).  Layout:
// geometry type (PxGeometryType: 0 sphere, 1 plane, 2 capsule, 3 box, 4 convex
// core with its core type in bits 8..15) and 4 floats per shape, poses 7 floats, contacts 8 floats (normal, separation,
// point, 0) with maxPerPair slots per pair.  Returns GBPX_ERR_CAPACITY if a
// pair produced more than maxPerPair contacts (counts are still exact).
static int generateContactsHost(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0, const float* pose1,
                                uint32_t nbPairs, float contactDistance, float toleranceLength, float* outContacts, uint32_t maxPerPair,
                                uint32_t* outCounts, void* manifolds)
{
	if(!nbPairs) return GBPX_OK;
	if(!type0 || !geom0 || !type1 || !geom1 || !pose0 || !pose1 || !outContacts || !outCounts || !maxPerPair) return GBPX_ERR_INVALID;
	if(!(contactDistance > 0.0f) || !(toleranceLength > 0.0f)) return GBPX_ERR_INVALID;
	uint32_t nbConvexCore = 0;
	for(uint32_t i = 0; i < nbPairs; i++)
	{
		if(!validShapeType(type0[i]) || !validShapeType(type1[i])) return GBPX_ERR_INVALID;
		if((type0[i] & 0xff) == 4 || (type1[i] & 0xff) == 4) nbConvexCore++;
	}
	NpWorkspace* ws = npWorkspace();
	if(!ws) return GBPX_ERR_CUDA;
	const size_t n = nbPairs;
	if(ws->t0.reserve(n) || ws->t1.reserve(n) || ws->g0.reserve(4 * n) || ws->g1.reserve(4 * n) || ws->p0.reserve(7 * n) ||
	   ws->p1.reserve(7 * n) || ws->hist.reserve(2 * np::NP_BINS) || ws->perm.reserve(n) || ws->counts.reserve(n) || ws->out.reserve(8 * n) ||
	   ws->hOut.reserve(8 * n) || ws->hCounts.reserve(n) || (manifolds && ws->manifolds.reserve(n)))
		return GBPX_ERR_NOMEM;
	cudaStream_t s = ws->stream;
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->t0.ptr, type0, n * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->t1.ptr, type1, n * 4, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->g0.ptr, geom0, n * 16, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->g1.ptr, geom1, n * 16, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->p0.ptr, pose0, n * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->p1.ptr, pose1, n * 28, cudaMemcpyHostToDevice, s));
	GBPX_CUDA_TRY(cudaMemsetAsync(ws->hist.ptr, 0, 2 * np::NP_BINS * 4, s));
	np::PairRef pr = {ws->t0.ptr, ws->g0.ptr, ws->t1.ptr, ws->g1.ptr, ws->p0.ptr, ws->p1.ptr};
	const uint32_t blocks = divUp(n, 256);
	np::bucketCountKernel<<<blocks, 256, 0, s>>>(pr, nbPairs, ws->hist.ptr);
	np::bucketOffsetsKernel<<<1, 32, 0, s>>>(ws->hist.ptr);
	np::bucketScatterKernel<<<blocks, 256, 0, s>>>(pr, nbPairs, ws->hist.ptr + np::NP_BINS, ws->perm.ptr);
	if(manifolds) GBPX_CUDA_TRY(cudaMemcpyAsync(ws->manifolds.ptr, manifolds, n * sizeof(np::ManifoldRecord), cudaMemcpyHostToDevice, s));
	// the convex-core pairs occupy the last nbConvexCore slots of the bucket order
	const uint32_t nbPrimitive = nbPairs - nbConvexCore;
	if(nbPrimitive)
		np::generateKernel<<<divUp(nbPrimitive, 128), 128, 0, s>>>(pr, ws->perm.ptr, nbPrimitive, contactDistance, toleranceLength, ws->out.ptr,
		                                                           ws->counts.ptr, manifolds ? ws->manifolds.ptr : nullptr);
	if(nbConvexCore)
		np::generateConvexCoreKernel<<<divUp(nbConvexCore, 128), 128, 0, s>>>(pr, ws->perm.ptr, nbPrimitive, nbPairs, contactDistance, ws->out.ptr,
		                                                                       ws->counts.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	if(manifolds) GBPX_CUDA_TRY(cudaMemcpyAsync(manifolds, ws->manifolds.ptr, n * sizeof(np::ManifoldRecord), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->hCounts.ptr, ws->counts.ptr, n * 4, cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ws->hOut.ptr, ws->out.ptr, n * 8 * sizeof(float4), cudaMemcpyDeviceToHost, s));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s));
	int rc = GBPX_OK;
	for(size_t i = 0; i < n; i++)
	{
		const uint32_t c = ws->hCounts.ptr[i];
		outCounts[i] = c;
		if(c > maxPerPair) rc = GBPX_ERR_CAPACITY;
		const uint32_t m = c < maxPerPair ? c : maxPerPair;
		memcpy(outContacts + i * maxPerPair * 8, ws->hOut.ptr + i * 8, size_t(m) * 8 * sizeof(float));
	}
	return rc;
}

GBPX_API int gbpx_generate_contacts(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                                    const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin,
                                    float toleranceLength, float* outContacts, uint32_t maxPerPair, uint32_t* outCounts)
{
	gbpx::Zone zone("gbpx::generateContacts");
	(void)meshContactMargin;
	return generateContactsHost(type0, geom0, type1, geom1, pose0, pose1, nbPairs, contactDistance, toleranceLength, outContacts, maxPerPair,
	                            outCounts, nullptr);
}

// PxGenerateContacts with persistent caches: manifolds (nbPairs x 288 bytes,
// host memory, all zero for a fresh cache) carries each pair's contact
// manifold from one call to the next, as PxCache does for the plane-capsule,
// plane-box, capsule-box and box-box pairs; it is read and updated.
GBPX_API int gbpx_generate_contacts_cached(const int* type0, const float* geom0, const int* type1, const float* geom1, const float* pose0,
                                           const float* pose1, uint32_t nbPairs, float contactDistance, float meshContactMargin,
                                           float toleranceLength, float* outContacts, uint32_t maxPerPair, uint32_t* outCounts, void* manifolds)
{
	gbpx::Zone zone("gbpx::generateContacts");
	(void)meshContactMargin;
	if(nbPairs && !manifolds) return GBPX_ERR_INVALID;
	return generateContactsHost(type0, geom0, type1, geom1, pose0, pose1, nbPairs, contactDistance, toleranceLength, outContacts, maxPerPair,
	                            outCounts, manifolds);
}

// ------------------------------------------------------------------ no-allocation variant
// The same narrowphase over caller-owned device arrays, with its bucketing
// scratch (the bin counters, the bin cursors and the pair permutation) in a
// fixed file-scope device array instead of per-call allocations.
namespace gbpx
{
constexpr uint32_t NP_NOALLOC_MAX_PAIRS = 262144;                  // 1 MiB of permutation
constexpr uint32_t NP_NOALLOC_SCRATCH_WORDS = 2 * np::NP_BINS + NP_NOALLOC_MAX_PAIRS;
static __device__ __align__(256) uint32_t gNpNoAllocScratch[NP_NOALLOC_SCRATCH_WORDS];
constexpr int NP_NOALLOC_MAX_DEVICES = 64;

// Address of the scratch array on the current device, looked up once per device
// (with that device current) by whichever host thread calls first; the other
// threads wait for that lookup.  The address belongs to the device's primary
// context, which the runtime API uses; a failed lookup is retried on the next
// call.
static int npNoAllocScratch(uint32_t** out)
{
	static std::atomic<uint32_t*> cache[NP_NOALLOC_MAX_DEVICES] = {};
	static std::mutex lookup;
	int dev = 0;
	GBPX_CUDA_TRY(cudaGetDevice(&dev));
	if(dev < 0 || dev >= NP_NOALLOC_MAX_DEVICES) return GBPX_ERR_INVALID;
	uint32_t* p = cache[dev].load(std::memory_order_acquire);
	if(!p)
	{
		std::lock_guard<std::mutex> g(lookup);
		p = cache[dev].load(std::memory_order_relaxed);
		if(!p)
		{
			void* addr = nullptr;
			GBPX_CUDA_TRY(cudaGetSymbolAddress(&addr, gNpNoAllocScratch));
			p = static_cast<uint32_t*>(addr);
			cache[dev].store(p, std::memory_order_release);
		}
	}
	*out = p;
	return GBPX_OK;
}
} // namespace gbpx

// PxGenerateContacts over nbPairs pairs held in device memory (layouts as
// gbpx_generate_contacts; contacts: 4 slots of 8 floats per pair, 16-byte
// aligned), enqueued on `stream` (a cudaStream_t, NULL for the default
// stream), with fresh caches.  Geometry types must be those of
// gbpx_generate_contacts (sphere, plane, capsule, box, convex core): the device
// arrays are not inspected on the host, and other values give undefined contacts.  Allocates nothing: the bucketing scratch is
// a fixed 1 MiB device array, so nbPairs is limited to 262144
// (GBPX_ERR_CAPACITY above).  The scratch is shared by all calls on a device:
// calls that may overlap (other streams, other host threads) race and must be
// serialised by the caller.  The first call on a device looks up the scratch
// address.
GBPX_API int gbpx_generate_contacts_device_noalloc(const int* dType0, const float* dGeom0, const int* dType1, const float* dGeom1,
                                                   const float* dPose0, const float* dPose1, uint32_t nbPairs, float contactDistance,
                                                   float toleranceLength, float* dOutContacts, uint32_t* dOutCounts, void* stream)
{
	gbpx::Zone zone("gbpx::generateContacts");
	if(!nbPairs) return GBPX_OK;
	if(!dType0 || !dGeom0 || !dType1 || !dGeom1 || !dPose0 || !dPose1 || !dOutContacts || !dOutCounts) return GBPX_ERR_INVALID;
	if(!(contactDistance > 0.0f) || !(toleranceLength > 0.0f)) return GBPX_ERR_INVALID;
	if(reinterpret_cast<uintptr_t>(dOutContacts) & 15u) return GBPX_ERR_INVALID;
	if(nbPairs > NP_NOALLOC_MAX_PAIRS) return GBPX_ERR_CAPACITY;
	uint32_t* scratch = nullptr;
	const int rc = npNoAllocScratch(&scratch);
	if(rc) return rc;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	// the bin counters start at zero; the cursors and the permutation are fully rewritten
	GBPX_CUDA_TRY(cudaMemsetAsync(scratch, 0, 2 * np::NP_BINS * 4, s));
	np::PairRef pr = {dType0, dGeom0, dType1, dGeom1, dPose0, dPose1};
	const uint32_t blocks = divUp(nbPairs, 256);
	uint32_t* perm = scratch + 2 * np::NP_BINS;
	np::bucketCountKernel<<<blocks, 256, 0, s>>>(pr, nbPairs, scratch);
	np::bucketOffsetsKernel<<<1, 32, 0, s>>>(scratch);
	np::bucketScatterKernel<<<blocks, 256, 0, s>>>(pr, nbPairs, scratch + np::NP_BINS, perm);
	// the split between the kinds is not known on the host: both generators cover
	// every slot and skip the other's pairs
	np::generateKernel<<<divUp(nbPairs, 128), 128, 0, s>>>(pr, perm, nbPairs, contactDistance, toleranceLength,
	                                                        reinterpret_cast<float4*>(dOutContacts), dOutCounts, nullptr);
	np::generateConvexCoreKernel<<<divUp(nbPairs, 128), 128, 0, s>>>(pr, perm, 0, nbPairs, contactDistance,
	                                                                  reinterpret_cast<float4*>(dOutContacts), dOutCounts);
	GBPX_CUDA_TRY(cudaGetLastError());
	return GBPX_OK;
}
