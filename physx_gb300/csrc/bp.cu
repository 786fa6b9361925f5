// Broadphase for the GB300 rigid-body step: a drop-in for PhysX's ABP
// PxBroadPhase (PxCreateBroadPhase(eABP) + update/fetchResults).
//
// Semantics follow the reference ABP (physx/source/lowlevelaabb/src/BpBroadPhaseABP.cpp):
//  * bounds are inflated by the per-object distance in float (BoxManager::prepareData,
//    :1712-1729), X extents are compared as order-preserving integer keys
//    (BpBroadPhaseIntegerAABB.h:44 encodeFloat), Y/Z as closed float intervals
//    (the SIMD test at :2216-2235);
//  * a pair is (re)tested only when at least one object was added/updated/removed
//    this frame; boxes that were not updated keep the bounds stored at their last
//    add/update (the reference's "sleeping" array);
//  * filtering is BpFiltering.h:90 groupFiltering with the LUT of BpFiltering.cpp:34;
//  * created/lost reporting follows ABP_PairManager::computeCreatedDeletedPairs (:3714):
//    new pairs are created, re-found pairs persist, pairs with an updated endpoint
//    that were not re-found are lost (reported unless an endpoint was removed), and
//    pairs between two non-updated objects persist silently.
//
// GB300 design: all object state lives in HBM indexed by handle; each update
// sorts the live boxes by their encoded min-X key with a hand-written radix
// sort, sweeps updated boxes warp-cooperatively (one ballot per 32
// candidates), and maintains the active pair set as a sorted array of 64-bit
// keys (id0 << 32 | id1, id0 < id1), so created/lost lists come out sorted and
// deterministic.
#include "common.cuh"
#include <chrono>
#include "bp_internal.h"
#include "radix_sort.cuh"
#include <vector>
#include <algorithm>

namespace gbpx
{
namespace bp
{
enum : uint8_t { F_UPDATED = 1, F_REMOVED = 2 };

// Packed add/update record staged on the host: id, group, distance, bounds.
struct UpdateRec
{
	uint32_t id;
	uint32_t group;
	float dist;
	float mn[3];
	float mx[3];
	uint32_t isCreate;
};
static_assert(sizeof(UpdateRec) == 40, "UpdateRec layout");

__device__ __forceinline__ bool lutAllows(uint32_t t0, uint32_t t1, uint32_t lutBits)
{
	return (lutBits >> (t0 * 7 + t1)) & 1u;
}

// The group filter's table row for a box of group g0: bit t1 set when a box of
// type t1 < 7 may pair with it (bit 7 stays clear, type 7 never pairs); zero for
// a box of type 7.  groupRowAllows(g0, groupRow(g0), g1) == groupFilter(g0, g1).
__device__ __forceinline__ uint32_t groupRow(uint32_t g0, uint32_t lutLo, uint32_t lutHi)
{
	const uint32_t t0 = g0 & 7u;
	if(t0 >= 7u) return 0u;
	const unsigned long long bits = (static_cast<unsigned long long>(lutHi) << 32) | lutLo;
	return uint32_t(bits >> (t0 * 7u)) & 0x7fu;
}

__device__ __forceinline__ bool groupRowAllows(uint32_t g0, uint32_t row, uint32_t g1)
{
	return (g0 != g1) & (((row >> (g1 & 7u)) & 1u) != 0u);
}

__device__ __forceinline__ bool groupFilter(uint32_t g0, uint32_t g1, uint32_t lutLo, uint32_t lutHi)
{
	if(g0 == g1) return false;
	const uint32_t t0 = g0 & 7u, t1 = g1 & 7u;
	if(t0 >= 7u || t1 >= 7u) return false;
	const uint32_t bit = t0 * 7u + t1;
	return bit < 32u ? ((lutLo >> bit) & 1u) : ((lutHi >> (bit - 32u)) & 1u);
}

__global__ void applyRemovedKernel(const uint32_t* __restrict__ ids, uint32_t n, uint8_t* __restrict__ live, uint8_t* __restrict__ flags)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const uint32_t id = ids[i];
	live[id] = 0;
	flags[id] = F_UPDATED | F_REMOVED;
}

__global__ void applyUpdatesKernel(const UpdateRec* __restrict__ recs, uint32_t n, uint2* __restrict__ bx, float4* __restrict__ byz,
                                   uint32_t* __restrict__ groups, uint8_t* __restrict__ live, uint8_t* __restrict__ flags)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const UpdateRec r = recs[i];
	const float d = r.dist;
	// Inflate exactly as the reference: min - d, max + d in FP32.
	const float minX = __fsub_rn(r.mn[0], d), minY = __fsub_rn(r.mn[1], d), minZ = __fsub_rn(r.mn[2], d);
	const float maxX = __fadd_rn(r.mx[0], d), maxY = __fadd_rn(r.mx[1], d), maxZ = __fadd_rn(r.mx[2], d);
	bx[r.id] = make_uint2(encodeFloatBits(__float_as_uint(minX)), encodeFloatBits(__float_as_uint(maxX)));
	byz[r.id] = make_float4(-minY, -minZ, maxY, maxZ);
	if(r.isCreate) groups[r.id] = r.group;
	live[r.id] = 1;
	flags[r.id] |= F_UPDATED;
}

// Bounds of handles [0, n) from device memory (6 floats each: min xyz, max xyz),
// distance 0: the large-scene step moves every dynamic body every frame.
__global__ void applyDeviceBoundsKernel(const float* __restrict__ bounds, uint32_t n, uint2* __restrict__ bx, float4* __restrict__ byz,
                                        uint8_t* __restrict__ flags)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const float* r = bounds + 6 * size_t(i);
	bx[i] = make_uint2(encodeFloatBits(__float_as_uint(r[0])), encodeFloatBits(__float_as_uint(r[3])));
	byz[i] = make_float4(-r[1], -r[2], r[4], r[5]);
	flags[i] |= F_UPDATED;
}

// Stable compaction of live handles into (key = encoded min X, value = handle).
__global__ void countLiveKernel(const uint8_t* __restrict__ live, uint32_t cap, uint32_t* __restrict__ blockCounts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = i < cap && live[i];
	const uint32_t b = __syncthreads_count(v);
	if(threadIdx.x == 0) blockCounts[blockIdx.x] = b;
}

__global__ void emitLiveKernel(const uint8_t* __restrict__ live, const uint2* __restrict__ bx, uint32_t cap,
                               const uint32_t* __restrict__ blockOffsets, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpCounts[32];
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = i < cap && live[i];
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t ballot = __ballot_sync(0xffffffffu, v);
	if(lane == 0) warpCounts[warp] = __popc(ballot);
	__syncthreads();
	if(warp == 0)
	{
		const uint32_t nw = blockDim.x >> 5;
		uint32_t c = lane < nw ? warpCounts[lane] : 0u;
		uint32_t incl = c;
		for(int o = 1; o < 32; o <<= 1)
		{
			const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
			if(lane >= uint32_t(o)) incl += t;
		}
		if(lane < nw) warpCounts[lane] = incl - c;
	}
	__syncthreads();
	if(v)
	{
		const uint32_t dst = blockOffsets[blockIdx.x] + warpCounts[warp] + __popc(ballot & laneMaskLt());
		keys[dst] = bx[i].x;
		vals[dst] = i;
	}
}

// Gathers the sorted SoA arrays and marks which sorted positions were updated.
// ---- sorted order, incremental (ABP's updated-only sort, BpBroadPhaseABP.cpp:1344,1484-1596):
// last frame's order without the removed and updated boxes is still sorted
// (their keys did not change); only the created / updated boxes are sorted, then
// the two lists are merged.  Equal keys put the kept box first; the order among
// equal keys changes no pair (a pair with an updated box is found once from
// whichever box comes first) and the found pairs are sorted afterwards.
__device__ __forceinline__ uint32_t lowerBound32(const uint32_t* __restrict__ arr, uint32_t n, uint32_t key)
{
	uint32_t a = 0, b = n;
	while(a < b)
	{
		const uint32_t m = (a + b) >> 1;
		if(arr[m] < key) a = m + 1; else b = m;
	}
	return a;
}
__device__ __forceinline__ uint32_t upperBound32(const uint32_t* __restrict__ arr, uint32_t n, uint32_t key)
{
	uint32_t a = 0, b = n;
	while(a < b)
	{
		const uint32_t m = (a + b) >> 1;
		if(arr[m] <= key) a = m + 1; else b = m;
	}
	return a;
}

// keep[i] = 1 for the boxes of last frame's order that are live and were not updated
__global__ void keepFlagKernel(const uint32_t* __restrict__ prevOrder, uint32_t n, const uint8_t* __restrict__ live,
                               const uint8_t* __restrict__ flags, uint32_t* __restrict__ keep)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const uint32_t id = prevOrder[i];
	keep[i] = (live[id] && !(flags[id] & F_UPDATED)) ? 1u : 0u;
}

// (key, handle) of the created / updated boxes: the update records' handles, or
// handles [0, n) (recs null: the device-bounds path)
__global__ void updatedKeysKernel(const UpdateRec* __restrict__ recs, uint32_t n, const uint2* __restrict__ bx, uint32_t* __restrict__ keys,
                                  uint32_t* __restrict__ vals)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n) return;
	const uint32_t id = recs ? recs[i].id : i;
	keys[i] = bx[id].x;
	vals[i] = id;
}

// kept handles and their keys, in last frame's order
__global__ void gatherKeptKernel(const uint32_t* __restrict__ prevOrder, const uint32_t* __restrict__ keptPos, uint32_t n,
                                 const uint2* __restrict__ bx, uint32_t* __restrict__ ids, uint32_t* __restrict__ keys)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
	if(j >= n) return;
	const uint32_t id = prevOrder[keptPos[j]];
	ids[j] = id;
	keys[j] = bx[id].x;
}

// Merge by co-ranking: the updated boxes after kept boxes of equal key.  Writes
// the merged order and the sorted positions of the updated (updPos) and kept
// (sleepPos) boxes, both ascending.
__global__ void mergeOrderKernel(const uint32_t* __restrict__ uKeys, const uint32_t* __restrict__ uIds, uint32_t nU,
                                 const uint32_t* __restrict__ sKeys, const uint32_t* __restrict__ sIds, uint32_t nS, uint32_t* __restrict__ order,
                                 uint32_t* __restrict__ updPos, uint32_t* __restrict__ sleepPos)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < nU)
	{
		const uint32_t pos = i + upperBound32(sKeys, nS, uKeys[i]);
		order[pos] = uIds[i];
		updPos[i] = pos;
	}
	else if(i < nU + nS)
	{
		const uint32_t j = i - nU;
		const uint32_t pos = j + lowerBound32(uKeys, nU, sKeys[j]);
		order[pos] = sIds[j];
		sleepPos[j] = pos;
	}
}

__global__ void gatherSortedKernel(const uint32_t* __restrict__ sortedIds, uint32_t n, const uint2* __restrict__ bx,
                                   const float4* __restrict__ byz, const uint32_t* __restrict__ groups, const uint8_t* __restrict__ flags,
                                   uint2* __restrict__ sx, float4* __restrict__ syz, uint32_t* __restrict__ sgrp, uint32_t* __restrict__ supd)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= n) return;
	const uint32_t id = sortedIds[p];
	sx[p] = bx[id];
	syz[p] = byz[id];
	sgrp[p] = groups[id];
	supd[p] = (flags[id] & F_UPDATED) ? 1u : 0u;
}

// Stable compaction of sorted positions that were / were not updated.
__global__ void countFlagKernel(const uint32_t* __restrict__ flag, uint32_t n, uint32_t want, uint32_t* __restrict__ blockCounts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = i < n && flag[i] == want;
	const uint32_t b = __syncthreads_count(v);
	if(threadIdx.x == 0) blockCounts[blockIdx.x] = b;
}

__global__ void emitFlagKernel(const uint32_t* __restrict__ flag, uint32_t n, uint32_t want, const uint32_t* __restrict__ blockOffsets,
                               uint32_t* __restrict__ out)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpCounts[32];
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = i < n && flag[i] == want;
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t ballot = __ballot_sync(0xffffffffu, v);
	if(lane == 0) warpCounts[warp] = __popc(ballot);
	__syncthreads();
	if(warp == 0)
	{
		const uint32_t nw = blockDim.x >> 5;
		uint32_t c = lane < nw ? warpCounts[lane] : 0u;
		uint32_t incl = c;
		for(int o = 1; o < 32; o <<= 1)
		{
			const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
			if(lane >= uint32_t(o)) incl += t;
		}
		if(lane < nw) warpCounts[lane] = incl - c;
	}
	__syncthreads();
	if(v) out[blockOffsets[blockIdx.x] + warpCounts[warp] + __popc(ballot & laneMaskLt())] = i;
}

__device__ __forceinline__ bool overlapYZ(const float4 a, const float4 b)
{
	// a, b hold (-minY, -minZ, maxY, maxZ): closed-interval overlap in Y and Z.
	return (b.x >= -a.z) & (b.y >= -a.w) & (b.z >= -a.x) & (b.w >= -a.y);
}

__device__ __forceinline__ void emitPairs(uint32_t hitMask, uint32_t idA, uint32_t idB, unsigned long long* __restrict__ out,
                                          uint32_t cap, uint32_t* __restrict__ counter)
{
	// Warp-aggregated append: one atomic per warp per batch of hits.
	const uint32_t lane = threadIdx.x & 31;
	if(!hitMask) return;
	uint32_t base = 0;
	if(lane == __ffs(hitMask) - 1) base = atomicAdd(counter, __popc(hitMask));
	base = __shfl_sync(0xffffffffu, base, __ffs(hitMask) - 1);
	if(hitMask & (1u << lane))
	{
		const uint32_t slot = base + __popc(hitMask & laneMaskLt());
		const uint32_t lo = min(idA, idB), hi = max(idA, idB);
		if(slot < cap) out[slot] = (static_cast<unsigned long long>(lo) << 32) | hi;
	}
}

// Pass 1: one warp per updated box; scans every later box in sorted order whose
// min X does not exceed this box's max X.
__global__ void sweepUpdatedKernel(const uint32_t* __restrict__ updPos, uint32_t nbUpd, uint32_t n, const uint2* __restrict__ sx,
                                   const float4* __restrict__ syz, const uint32_t* __restrict__ sgrp, const uint32_t* __restrict__ sortedIds,
                                   uint32_t lutLo, uint32_t lutHi, unsigned long long* __restrict__ out, uint32_t cap, uint32_t* __restrict__ counter)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t warpId = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nWarps = (gridDim.x * blockDim.x) >> 5;
	for(uint32_t k = warpId; k < nbUpd; k += nWarps)
	{
		const uint32_t p = updPos[k];
		const uint2 x0 = sx[p];
		const float4 yz0 = syz[p];
		const uint32_t g0 = sgrp[p];
		const uint32_t id0 = sortedIds[p];
		for(uint32_t q0 = p + 1; q0 < n; q0 += 32)
		{
			const uint32_t q = q0 + lane;
			bool inRange = false, hit = false;
			if(q < n)
			{
				inRange = sx[q].x <= x0.y;
				if(inRange) hit = overlapYZ(yz0, syz[q]) && groupFilter(g0, sgrp[q], lutLo, lutHi);
			}
			const uint32_t hitMask = __ballot_sync(0xffffffffu, hit);
			emitPairs(hitMask, id0, q < n ? sortedIds[q] : 0u, out, cap, counter);
			if(__ballot_sync(0xffffffffu, inRange) != 0xffffffffu) break;
		}
	}
}

// Pass 2: one thread per non-updated box; scans the updated boxes that come
// later in sorted order (pairs whose first box in sorted order did not move).
// A box whose X range covers more than SLEEP_SCAN_MAX updated boxes (a static
// ground plane covers all of them) is handed to sweepLongKernel as (box, first,
// end, first chunk) so that no thread runs a long serial scan: its candidates
// are cut into chunks of LONG_CHUNK that any block may take.
constexpr uint32_t SLEEP_SCAN_MAX = 256;
constexpr uint32_t LONG_CHUNK = 1024;
__global__ void sweepSleepingKernel(const uint32_t* __restrict__ sleepPos, uint32_t nbSleep, const uint32_t* __restrict__ updPos,
                                    uint32_t nbUpd, const uint2* __restrict__ sx, const float4* __restrict__ syz,
                                    const uint32_t* __restrict__ sgrp, const uint32_t* __restrict__ sortedIds, uint32_t lutLo,
                                    uint32_t lutHi, unsigned long long* __restrict__ out, uint32_t cap, uint32_t* __restrict__ counter,
                                    uint4* __restrict__ longScans, unsigned long long* __restrict__ longCount)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t lane = threadIdx.x & 31;
	uint32_t p = 0, lo = nbUpd;
	uint2 x0 = make_uint2(1u, 0u);
	float4 yz0 = make_float4(0, 0, 0, 0);
	uint32_t g0 = 0, id0 = 0;
	const bool active = k < nbSleep;
	if(active)
	{
		p = sleepPos[k];
		x0 = sx[p];
		yz0 = syz[p];
		g0 = sgrp[p];
		id0 = sortedIds[p];
		// first updated position > p
		uint32_t a = 0, b = nbUpd;
		while(a < b)
		{
			const uint32_t m = (a + b) >> 1;
			if(updPos[m] <= p) a = m + 1; else b = m;
		}
		lo = a;
		// end of the candidates: updated boxes' min X keys ascend with their position
		b = nbUpd;
		while(a < b)
		{
			const uint32_t m = (a + b) >> 1;
			if(sx[updPos[m]].x <= x0.y) a = m + 1; else b = m;
		}
		if(a - lo > SLEEP_SCAN_MAX)
		{
			// one atomic counts the item (high word) and its chunks (low word), so the
			// items are numbered in increasing order of their first chunk
			const unsigned long long chunks = (a - lo + LONG_CHUNK - 1) / LONG_CHUNK;
			const unsigned long long old = atomicAdd(longCount, (1ull << 32) | chunks);
			longScans[uint32_t(old >> 32)] = make_uint4(p, lo, a, uint32_t(old));
			lo = nbUpd;
		}
	}
	bool more = active && lo < nbUpd;
	uint32_t j = lo;
	while(__any_sync(0xffffffffu, more))
	{
		bool hit = false;
		uint32_t idq = 0;
		if(more)
		{
			const uint32_t q = updPos[j];
			if(sx[q].x <= x0.y)
			{
				idq = sortedIds[q];
				hit = overlapYZ(yz0, syz[q]) && groupFilter(g0, sgrp[q], lutLo, lutHi);
				j++;
				more = j < nbUpd;
			}
			else more = false;
		}
		// Emission is per lane here (divergent scans); aggregate the lanes that hit.
		const uint32_t hitMask = __ballot_sync(0xffffffffu, hit);
		if(hitMask)
		{
			uint32_t base = 0;
			const uint32_t leader = __ffs(hitMask) - 1;
			if(lane == leader) base = atomicAdd(counter, __popc(hitMask));
			base = __shfl_sync(0xffffffffu, base, leader);
			if(hit)
			{
				const uint32_t slot = base + __popc(hitMask & laneMaskLt());
				const uint32_t a = min(id0, idq), b = max(id0, idq);
				if(slot < cap) out[slot] = (static_cast<unsigned long long>(a) << 32) | b;
			}
		}
	}
}

// The long scans of pass 2: warps take chunks of LONG_CHUNK candidates of any
// item (its box against updated boxes [first, end)), lanes striding over a chunk.
// The item holding chunk g (the last whose first chunk is <= g) is found by a
// 32-way search: each step the lanes probe 32 evenly spaced items.
__global__ void __launch_bounds__(256) sweepLongKernel(const uint4* __restrict__ longScans, const unsigned long long* __restrict__ longCount,
                                                       const uint32_t* __restrict__ updPos, const uint2* __restrict__ sx,
                                                       const float4* __restrict__ syz, const uint32_t* __restrict__ sgrp,
                                                       const uint32_t* __restrict__ sortedIds, uint32_t lutLo, uint32_t lutHi,
                                                       unsigned long long* __restrict__ out, uint32_t cap, uint32_t* __restrict__ counter)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const unsigned long long lc = *longCount;
	const uint32_t items = uint32_t(lc >> 32), chunks = uint32_t(lc);
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t warpId = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nWarps = (gridDim.x * blockDim.x) >> 5;
	for(uint32_t g = warpId; g < chunks; g += nWarps)
	{
		// invariant: longScans[a].w <= g, and b == items or longScans[b].w > g
		uint32_t a = 0, b = items;
		while(b - a > 32)
		{
			const uint32_t step = (b - a + 31) / 32;
			const uint32_t idx = a + lane * step;
			const bool le = idx < b && longScans[idx].w <= g;
			const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, le));   // a prefix of the lanes
			a += (cnt - 1) * step;
			b = min(b, a + step);
		}
		const bool le = a + lane < b && longScans[a + lane].w <= g;
		a += __popc(__ballot_sync(0xffffffffu, le)) - 1;
		const uint4 ls = longScans[a];
		const uint32_t p = ls.x;
		const float4 yz0 = syz[p];
		const uint32_t g0 = sgrp[p], row = groupRow(g0, lutLo, lutHi);
		const uint32_t id0 = sortedIds[p];
		const uint32_t first = ls.y + (g - ls.w) * LONG_CHUNK, end = min(ls.z, first + LONG_CHUNK);
		for(uint32_t u0 = first; u0 < end; u0 += 32)
		{
			const uint32_t u = u0 + lane;
			bool hit = false;
			uint32_t idq = 0;
			if(u < end)
			{
				const uint32_t q = updPos[u];
				hit = overlapYZ(yz0, syz[q]) && groupRowAllows(g0, row, sgrp[q]);
				if(hit) idq = sortedIds[q];
			}
			emitPairs(__ballot_sync(0xffffffffu, hit), id0, idq, out, cap, counter);
		}
	}
}

// Pass 1, tiled: a block takes UPD_PER_BLOCK consecutive updated boxes (in
// sorted order, so their candidate ranges overlap) and streams the union of the
// ranges through shared memory in tiles of SWEEP_TILE sorted positions; each
// warp tests its UPD_PER_WARP boxes against each tile, lanes striding over the
// positions.  The end of a box's range within the tile (the first later position
// whose min X is past its max X) is found first by a 32-way search of the
// tile's min X keys, which ascend.  The candidates are read from memory about
// once per block instead of once per box, and tiles that no unfinished box
// reaches are skipped.  Finds the same pairs as sweepUpdatedKernel.
constexpr uint32_t UPD_PER_WARP = 8;
constexpr uint32_t UPD_PER_BLOCK = 8 * UPD_PER_WARP;   // 8 warps
constexpr uint32_t SWEEP_TILE = 1024;
__global__ void __launch_bounds__(256) sweepUpdatedTiledKernel(const uint32_t* __restrict__ updPos, uint32_t nbUpd, uint32_t n,
                                                               const uint2* __restrict__ sx, const float4* __restrict__ syz,
                                                               const uint32_t* __restrict__ sgrp, const uint32_t* __restrict__ sortedIds,
                                                               uint32_t lutLo, uint32_t lutHi, unsigned long long* __restrict__ out, uint32_t cap,
                                                               uint32_t* __restrict__ counter)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t tMinX[SWEEP_TILE], tGrp[SWEEP_TILE], tId[SWEEP_TILE];
	__shared__ float4 tYZ[SWEEP_TILE];
	__shared__ uint32_t warpNext[8];
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for(uint32_t blk = blockIdx.x; blk * UPD_PER_BLOCK < nbUpd; blk += gridDim.x)
	{
		const uint32_t k0 = blk * UPD_PER_BLOCK;
		// lane j < UPD_PER_WARP holds box k0 + warp * UPD_PER_WARP + j
		const uint32_t kb = k0 + warp * UPD_PER_WARP + lane;
		bool pending = lane < UPD_PER_WARP && kb < nbUpd;
		uint32_t bp = 0, bMaxX = 0, bGrp = 0, bRow = 0, bId = 0;
		float4 bYZ = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		if(pending)
		{
			bp = updPos[kb];
			bMaxX = sx[bp].y;
			bYZ = syz[bp];
			bGrp = sgrp[bp];
			bRow = groupRow(bGrp, lutLo, lutHi);
			bId = sortedIds[bp];
			pending = bp + 1 < n;
		}
		uint32_t tileStart = updPos[k0] + 1;   // updPos ascends: the block's first box comes first
		while(tileStart < n)
		{
			const uint32_t tileEnd = min(n, tileStart + SWEEP_TILE);
			__syncthreads();
			for(uint32_t i = threadIdx.x; tileStart + i < tileEnd; i += blockDim.x)
			{
				const uint32_t q = tileStart + i;
				tMinX[i] = sx[q].x;
				tYZ[i] = syz[q];
				tGrp[i] = sgrp[q];
				tId[i] = sortedIds[q];
			}
			__syncthreads();
			for(uint32_t j = 0; j < UPD_PER_WARP; j++)
			{
				if(!__shfl_sync(0xffffffffu, pending ? 1u : 0u, j)) continue;
				const uint32_t p = __shfl_sync(0xffffffffu, bp, j);
				const uint32_t first = max(p + 1, tileStart);
				if(first >= tileEnd) continue;
				const uint32_t maxX = __shfl_sync(0xffffffffu, bMaxX, j);
				// end of the range in this tile: positions in [a, end) are in range, [end, b) are not
				uint32_t a = first, b = tileEnd;
				while(b - a > 32)
				{
					const uint32_t step = (b - a + 31) >> 5;
					const uint32_t idx = a + lane * step;
					const bool le = idx < b && tMinX[idx - tileStart] <= maxX;
					const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, le));   // a prefix of the lanes
					if(cnt == 0) { b = a; break; }
					const uint32_t hiB = a + cnt * step;
					a += (cnt - 1) * step + 1;
					b = min(b, hiB);
				}
				const uint32_t end = a + __popc(__ballot_sync(0xffffffffu, a + lane < b && tMinX[min(a + lane, tileEnd - 1) - tileStart] <= maxX));
				if(end < tileEnd && lane == j) pending = false;   // the range ends inside this tile
				if(end <= first) continue;
				const uint32_t g0 = __shfl_sync(0xffffffffu, bGrp, j), row = __shfl_sync(0xffffffffu, bRow, j);
				const uint32_t id0 = __shfl_sync(0xffffffffu, bId, j);
				const float4 yz0 = make_float4(__shfl_sync(0xffffffffu, bYZ.x, j), __shfl_sync(0xffffffffu, bYZ.y, j),
				                               __shfl_sync(0xffffffffu, bYZ.z, j), __shfl_sync(0xffffffffu, bYZ.w, j));
				for(uint32_t q0 = first; q0 < end; q0 += 32)
				{
					const uint32_t q = q0 + lane;
					bool hit = false;
					uint32_t idq = 0;
					if(q < end)
					{
						const uint32_t i = q - tileStart;
						hit = overlapYZ(yz0, tYZ[i]) && groupRowAllows(g0, row, tGrp[i]);
						if(hit) idq = tId[i];
					}
					const uint32_t hm = __ballot_sync(0xffffffffu, hit);
					if(hm) emitPairs(hm, id0, idq, out, cap, counter);
				}
			}
			// next tile: the smallest position an unfinished box still has to scan
			uint32_t next = pending ? max(bp + 1, tileEnd) : 0xffffffffu;
			next = __reduce_min_sync(0xffffffffu, next);
			if(lane == 0) warpNext[warp] = next;
			__syncthreads();
			next = warpNext[0];
			for(uint32_t w = 1; w < 8; w++) next = min(next, warpNext[w]);
			tileStart = next;   // all ones when every box is done
		}
	}
}

// Pass 2, tiled: a block takes SLEEP_PER_BLOCK consecutive non-updated boxes (in
// sorted order), one per thread.  Each finds its candidates (updated boxes later
// in sorted order whose min X is within its X range) as sweepSleepingKernel does,
// handing a range longer than SLEEP_SCAN_MAX to the long-scan list.  The updated
// boxes of the union of the block's ranges are gathered into shared memory a tile
// at a time; each warp then takes its 32 boxes one after another, lanes striding
// over the box's candidates in the tile.  Finds the same pairs as
// sweepSleepingKernel.
constexpr uint32_t SLEEP_PER_BLOCK = 256;
constexpr uint32_t SLEEP_TILE = 1024;
struct SleepBox
{
	float4 yz;
	uint32_t lo, hi, grp, id;
};
__global__ void __launch_bounds__(256) sweepSleepingTiledKernel(const uint32_t* __restrict__ sleepPos, uint32_t nbSleep,
                                                                const uint32_t* __restrict__ updPos, uint32_t nbUpd,
                                                                const uint2* __restrict__ sx, const float4* __restrict__ syz,
                                                                const uint32_t* __restrict__ sgrp, const uint32_t* __restrict__ sortedIds,
                                                                uint32_t lutLo, uint32_t lutHi, unsigned long long* __restrict__ out, uint32_t cap,
                                                                uint32_t* __restrict__ counter, uint4* __restrict__ longScans,
                                                                unsigned long long* __restrict__ longCount)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t tGrp[SLEEP_TILE], tId[SLEEP_TILE];
	__shared__ float4 tYZ[SLEEP_TILE];
	__shared__ SleepBox boxes[SLEEP_PER_BLOCK];
	__shared__ uint32_t sLo, sHi;
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for(uint32_t blk = blockIdx.x; blk * SLEEP_PER_BLOCK < nbSleep; blk += gridDim.x)
	{
		const uint32_t k = blk * SLEEP_PER_BLOCK + threadIdx.x;
		__syncthreads();   // the previous box set is done with the shared state
		if(threadIdx.x == 0) { sLo = 0xffffffffu; sHi = 0; }
		__syncthreads();
		SleepBox box{make_float4(0.0f, 0.0f, 0.0f, 0.0f), 0u, 0u, 0u, 0u};
		if(k < nbSleep)
		{
			const uint32_t p = sleepPos[k];
			const uint2 x0 = sx[p];
			box.yz = syz[p];
			box.grp = sgrp[p];
			box.id = sortedIds[p];
			// sleepPos and updPos partition the sorted positions, both ascending: the
			// updated boxes before position p number p - k
			const uint32_t lo = p - k;
			// end of the candidates (their min X ascends with the position), searched
			// within SLEEP_SCAN_MAX + 1 of lo unless the range is a long one
			uint32_t a = lo, b = min(nbUpd, lo + SLEEP_SCAN_MAX + 1);
			if(b == lo + SLEEP_SCAN_MAX + 1 && sx[updPos[b - 1]].x <= x0.y) { a = b; b = nbUpd; }
			while(a < b)
			{
				const uint32_t m = (a + b) >> 1;
				if(sx[updPos[m]].x <= x0.y) a = m + 1; else b = m;
			}
			uint32_t hi = a;
			if(hi - lo > SLEEP_SCAN_MAX)
			{
				const unsigned long long chunks = (hi - lo + LONG_CHUNK - 1) / LONG_CHUNK;
				const unsigned long long old = atomicAdd(longCount, (1ull << 32) | chunks);
				longScans[uint32_t(old >> 32)] = make_uint4(p, lo, hi, uint32_t(old));
				hi = lo;
			}
			box.lo = lo;
			box.hi = hi;
			if(hi > lo)
			{
				atomicMin(&sLo, lo);
				atomicMax(&sHi, hi);
			}
		}
		boxes[threadIdx.x] = box;
		__syncthreads();
		const uint32_t uLo = sLo, uHi = sHi;
		for(uint32_t t0 = uLo; t0 < uHi; t0 += SLEEP_TILE)
		{
			const uint32_t t1 = min(uHi, t0 + SLEEP_TILE);
			for(uint32_t i = threadIdx.x; t0 + i < t1; i += blockDim.x)
			{
				const uint32_t q = updPos[t0 + i];
				tYZ[i] = syz[q];
				tGrp[i] = sgrp[q];
				tId[i] = sortedIds[q];
			}
			__syncthreads();
			for(uint32_t j = 0; j < 32; j++)
			{
				const SleepBox& bx = boxes[warp * 32 + j];
				const uint32_t a = max(bx.lo, t0), b = min(bx.hi, t1);
				if(a >= b) continue;
				const float4 yz0 = bx.yz;
				const uint32_t g0 = bx.grp, id0 = bx.id, row = groupRow(g0, lutLo, lutHi);
				for(uint32_t u0 = a; u0 < b; u0 += 32)
				{
					const uint32_t u = u0 + lane;
					bool hit = false;
					uint32_t idq = 0;
					if(u < b)
					{
						const uint32_t i = u - t0;
						hit = overlapYZ(yz0, tYZ[i]) && groupRowAllows(g0, row, tGrp[i]);
						if(hit) idq = tId[i];
					}
					const uint32_t hm = __ballot_sync(0xffffffffu, hit);
					if(hm) emitPairs(hm, id0, idq, out, cap, counter);
				}
			}
			__syncthreads();
		}
	}
}

__device__ __forceinline__ bool containsKey(const unsigned long long* __restrict__ arr, uint32_t n, unsigned long long key)
{
	uint32_t a = 0, b = n;
	while(a < b)
	{
		const uint32_t m = (a + b) >> 1;
		if(arr[m] < key) a = m + 1; else b = m;
	}
	return a < n && arr[a] == key;
}

__device__ __forceinline__ uint32_t lowerBound(const unsigned long long* __restrict__ arr, uint32_t n, unsigned long long key)
{
	uint32_t a = 0, b = n;
	while(a < b)
	{
		const uint32_t m = (a + b) >> 1;
		if(arr[m] < key) a = m + 1; else b = m;
	}
	return a;
}

// Classifies found pairs: flag 1 = created (absent from the previous set).
__global__ void classifyFoundKernel(const unsigned long long* __restrict__ found, uint32_t nFound, const unsigned long long* __restrict__ prev,
                                    uint32_t nPrev, uint32_t* __restrict__ isCreated)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nFound) return;
	isCreated[i] = containsKey(prev, nPrev, found[i]) ? 0u : 1u;
}

// Classifies previous pairs: 0 = persists via the found set, 1 = kept (both
// endpoints sleeping), 2 = lost and reported, 3 = dropped silently (removed endpoint).
__global__ void classifyPrevKernel(const unsigned long long* __restrict__ prev, uint32_t nPrev, const unsigned long long* __restrict__ found,
                                   uint32_t nFound, const uint8_t* __restrict__ flags, uint32_t* __restrict__ cls)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nPrev) return;
	const unsigned long long k = prev[i];
	const uint32_t id0 = uint32_t(k >> 32), id1 = uint32_t(k);
	const uint8_t f0 = flags[id0], f1 = flags[id1];
	uint32_t c;
	if(!((f0 | f1) & F_UPDATED)) c = 1;
	else if(containsKey(found, nFound, k)) c = 0;
	else if((f0 | f1) & F_REMOVED) c = 3;
	else c = 2;
	cls[i] = c;
}

__global__ void flagEqualsKernel(const uint32_t* __restrict__ cls, uint32_t n, uint32_t want, uint32_t* __restrict__ out)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) out[i] = cls[i] == want ? 1u : 0u;
}

__global__ void scatterSelectedKernel(const unsigned long long* __restrict__ src, const uint32_t* __restrict__ sel,
                                      const uint32_t* __restrict__ pos, uint32_t n, unsigned long long* __restrict__ dst)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n && sel[i]) dst[pos[i]] = src[i];
}

// Merge of two sorted, disjoint key arrays by co-ranking, the first one's length
// read from device memory: threads [0, keepCap) place its keys (those below
// *nKeep), threads [keepCap, keepCap + nb) the second's; thread 0 also writes the
// merged count to *nOut.
__global__ void mergeCountedKernel(const unsigned long long* __restrict__ a, const uint32_t* __restrict__ nKeep, uint32_t keepCap,
                                   const unsigned long long* __restrict__ b, uint32_t nb, unsigned long long* __restrict__ out, uint32_t* __restrict__ nOut)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t na = *nKeep;
	if(i == 0) *nOut = na + nb;
	if(i < keepCap)
	{
		if(i < na) out[i + lowerBound(b, nb, a[i])] = a[i];
	}
	else if(i < keepCap + nb)
	{
		const uint32_t j = i - keepCap;
		out[j + lowerBound(a, na, b[j])] = b[j];
	}
}

// Pair keys (id0 << 32 | id1) to (id0, id1) for the first *n keys; the grid is
// sized by an upper bound of *n.
__global__ void keysToPairsCountedKernel(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ n, uint2* __restrict__ out)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < *n) out[i] = make_uint2(uint32_t(keys[i] >> 32), uint32_t(keys[i]));
}

} // namespace bp

// One ABP-compatible broadphase instance.
struct BroadPhase
{
	cudaStream_t stream = 0;
	uint32_t lutLo = 0, lutHi = 0;
	uint32_t capacity = 0;  // handle capacity on device

	DevBuf<uint2> bx;
	DevBuf<float4> byz;
	DevBuf<uint32_t> groups;
	DevBuf<uint8_t> live, flags;

	// per-update scratch
	DevBuf<bp::UpdateRec> dRecs;
	DevBuf<uint32_t> dRemoved;
	HostBuf<bp::UpdateRec> hRecs;
	DevBuf<uint32_t> blockCounts, keysA, valsA, keysB, valsB, hist, scanScratch;
	DevBuf<uint2> sx;
	DevBuf<float4> syz;
	DevBuf<uint32_t> sgrp, supd, updPos, sleepPos;
	// the sorted order of the live boxes, kept from frame to frame (two sides)
	DevBuf<uint32_t> order[2], keepFlag, keptPos, keptIds, keptKeys;
	uint32_t orderSide = 0, nOrder = 0;
	DevBuf<unsigned long long> found, foundAlt, prev, next, created, lost;
	DevBuf<uint32_t> counter, cls, sel, pos;
	DevBuf<uint4> longScans;
	HostBuf<uint32_t> hCounts;
	HostBuf<uint2> hCreated, hLost;
	uint32_t nPrev = 0;
	uint32_t nbCreatedOut = 0, nbLostOut = 0;
	// created, lost, kept and next-active counts of the frame in flight, on the device
	// and (after the frame's one synchronisation) in pinned host memory
	DevBuf<uint32_t> frameCounts;
	HostBuf<uint32_t> hFrameCounts;
	uint32_t nFoundLast = 0;
	bool pending = false;
	uint64_t stats[4] = {0, 0, 0, 0};  // live boxes, updated boxes, found pairs, active pairs (last update)
	// timing of the last update: host staging of the user's arrays (ms), and the
	// device work from the first upload to the results in host memory (CUDA events)
	float lastHostMs = 0.0f, lastDeviceMs = 0.0f;
	int sweepTiled = 1;   // 1: shared-memory tiled sweeps, 0: one warp / thread per box
	cudaEvent_t evBegin = nullptr, evEnd = nullptr;

	int init(bool discardStaticKinematic, bool discardKinematicKinematic)
	{
		// LUT of BpFiltering.cpp:34 (7 filter types), flattened type0*7+type1.
		bool lut[7][7] = {};
		const int S = 0, K = 1, D = 2, A = 3, DS = 4, DV = 5, PS = 6;
		auto set = [&](int a, int b, bool v) { lut[a][b] = lut[b][a] = v; };
		set(S, D, true);
		set(S, K, !discardStaticKinematic);
		set(D, K, true);
		set(D, D, true);
		set(K, K, !discardKinematicKinematic);
		set(S, A, true); set(K, A, true); set(D, A, true); set(A, A, true);
		set(DS, D, true); set(DS, S, true); set(DS, K, true); set(DS, DS, true);
		set(DV, D, true); set(DV, S, true); set(DV, K, true); set(DV, DS, true); set(DV, DV, true);
		set(PS, D, true); set(PS, S, true); set(PS, K, true); set(PS, DS, true); set(PS, DV, true); set(PS, PS, true);
		uint64_t bits = 0;
		for(int a = 0; a < 7; a++)
			for(int b = 0; b < 7; b++)
				if(lut[a][b]) bits |= 1ull << (a * 7 + b);
		lutLo = uint32_t(bits);
		lutHi = uint32_t(bits >> 32);
		GBPX_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
		if(counter.reserve(4)) return GBPX_ERR_NOMEM;
		if(hCounts.reserve(8)) return GBPX_ERR_NOMEM;
		return GBPX_OK;
	}

	void release()
	{
		if(stream) cudaStreamSynchronize(stream);
		bx.release(); byz.release(); groups.release(); live.release(); flags.release();
		dRecs.release(); dRemoved.release(); hRecs.release();
		blockCounts.release(); scanScratch.release(); keysA.release(); valsA.release(); keysB.release(); valsB.release(); hist.release();
		sx.release(); syz.release(); sgrp.release(); supd.release(); updPos.release(); sleepPos.release();
		order[0].release(); order[1].release(); keepFlag.release(); keptPos.release(); keptIds.release(); keptKeys.release();
		found.release(); foundAlt.release(); prev.release(); next.release(); created.release(); lost.release();
		counter.release(); cls.release(); sel.release(); pos.release(); frameCounts.release(); longScans.release();
		hCounts.release(); hCreated.release(); hLost.release(); hFrameCounts.release();
		if(evBegin) cudaEventDestroy(evBegin);
		if(evEnd) cudaEventDestroy(evEnd);
		evBegin = evEnd = nullptr;
		if(stream) cudaStreamDestroy(stream);
		stream = 0;
	}

	int growCapacity(uint32_t need)
	{
		if(need <= capacity) return GBPX_OK;
		uint32_t nc = capacity ? capacity : 1024;
		while(nc < need) nc *= 2;
		DevBuf<uint2> nbx; DevBuf<float4> nbyz; DevBuf<uint32_t> ng; DevBuf<uint8_t> nl, nf;
		if(nbx.reserve(nc) || nbyz.reserve(nc) || ng.reserve(nc) || nl.reserve(nc) || nf.reserve(nc)) return GBPX_ERR_NOMEM;
		GBPX_CUDA_TRY(cudaMemsetAsync(nl.ptr, 0, nc, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(nf.ptr, 0, nc, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(ng.ptr, 0xff, size_t(nc) * 4, stream));
		if(capacity)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(nbx.ptr, bx.ptr, size_t(capacity) * sizeof(uint2), cudaMemcpyDeviceToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(nbyz.ptr, byz.ptr, size_t(capacity) * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(ng.ptr, groups.ptr, size_t(capacity) * 4, cudaMemcpyDeviceToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(nl.ptr, live.ptr, capacity, cudaMemcpyDeviceToDevice, stream));
		}
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		bx.release(); byz.release(); groups.release(); live.release(); flags.release();
		bx = nbx; byz = nbyz; groups = ng; live = nl; flags = nf;
		capacity = nc;
		return GBPX_OK;
	}

	// Compacts sorted positions p with flag[p] == want into out (stable).
	int compactFlag(const uint32_t* flag, uint32_t n, uint32_t want, uint32_t* out)
	{
		const uint32_t nb = divUp(n, 256);
		if(blockCounts.reserve(nb + 1)) return GBPX_ERR_NOMEM;
		(void)launchDependent(bp::countFlagKernel, nb, 256, stream, flag, n, want, blockCounts.ptr);
		if(cudaMemsetAsync(blockCounts.ptr + nb, 0, 4, stream) != cudaSuccess) return GBPX_ERR_CUDA;
		(void)launchDependent(rs::scanKernel, 1, 1024, stream, blockCounts.ptr, nb + 1);
		(void)launchDependent(bp::emitFlagKernel, nb, 256, stream, flag, n, want, blockCounts.ptr, out);
		return GBPX_OK;
	}

	// Exclusive scan of sel[0..n) into pos (total at pos[n]), copied to *countOut on
	// the device; nothing waits for it.
	int scanToDevice(const uint32_t* selIn, uint32_t n, uint32_t* posOut, uint32_t* countOut)
	{
		GBPX_CUDA_TRY(cudaMemcpyAsync(posOut, selIn, size_t(n) * 4, cudaMemcpyDeviceToDevice, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(posOut + n, 0, 4, stream));
		if(scanScratch.reserve(rs::scanScratchEntries(n + 1))) return GBPX_ERR_NOMEM;
		rs::scanAny(posOut, n + 1, scanScratch.ptr, stream);
		GBPX_CUDA_TRY(cudaMemcpyAsync(countOut, posOut + n, 4, cudaMemcpyDeviceToDevice, stream));
		return GBPX_OK;
	}

	// The host side of the frame once its stream has drained: counts in force.
	void finishFrame()
	{
		nbCreatedOut = hFrameCounts.ptr[0];
		nbLostOut = hFrameCounts.ptr[1];
		nPrev = hFrameCounts.ptr[3];
		stats[3] = nPrev;
	}

	int update(const uint32_t* createdIds, uint32_t nbCreated, const uint32_t* updatedIds, uint32_t nbUpdated,
	           const uint32_t* removedIds, uint32_t nbRemoved, const float* bounds, const uint32_t* groupsIn,
	           const float* distances, uint32_t cap)
	{
		if(pending) return GBPX_ERR_STATE;
		if((nbCreated && !createdIds) || (nbUpdated && !updatedIds) || (nbRemoved && !removedIds)) return GBPX_ERR_INVALID;
		if((nbCreated || nbUpdated) && (!bounds || !distances)) return GBPX_ERR_INVALID;
		if(nbCreated && !groupsIn) return GBPX_ERR_INVALID;
		for(uint32_t i = 0; i < nbCreated; i++) if(createdIds[i] >= cap) return GBPX_ERR_INVALID;
		for(uint32_t i = 0; i < nbUpdated; i++) if(updatedIds[i] >= cap) return GBPX_ERR_INVALID;
		for(uint32_t i = 0; i < nbRemoved; i++) if(removedIds[i] >= capacity) return GBPX_ERR_INVALID;
		int rc = growCapacity(cap);
		if(rc) return rc;

		// 1. Stage add/update records (host gather of the user-owned arrays) and upload.
		const uint32_t nbRec = nbCreated + nbUpdated;
		if(hRecs.reserve(nbRec ? nbRec : 1) || dRecs.reserve(nbRec ? nbRec : 1) || dRemoved.reserve(nbRemoved ? nbRemoved : 1))
			return GBPX_ERR_NOMEM;
		const auto hostBegin = std::chrono::steady_clock::now();
		auto gather = [&](uint32_t begin, uint32_t end) {
			for(uint32_t i = begin; i < end; i++)
			{
				const bool isC = i < nbCreated;
				const uint32_t id = isC ? createdIds[i] : updatedIds[i - nbCreated];
				bp::UpdateRec& r = hRecs.ptr[i];
				r.id = id;
				r.group = isC ? groupsIn[id] : 0u;
				r.dist = distances[id];
				memcpy(r.mn, bounds + 6 * size_t(id), 12);
				memcpy(r.mx, bounds + 6 * size_t(id) + 3, 12);
				r.isCreate = isC ? 1u : 0u;
			}
		};
		// the gather reads the user's arrays at random handles: large batches are
		// split over the host worker pool
		if(nbRec >= (1u << 15)) hostParallelFor(nbRec, 4096, gather);
		else gather(0, nbRec);
		lastHostMs = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - hostBegin).count();
		if(!evBegin) GBPX_CUDA_TRY(cudaEventCreate(&evBegin));
		if(!evEnd) GBPX_CUDA_TRY(cudaEventCreate(&evEnd));
		GBPX_CUDA_TRY(cudaEventRecord(evBegin, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, capacity, stream));
		if(nbRemoved)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(dRemoved.ptr, removedIds, size_t(nbRemoved) * 4, cudaMemcpyHostToDevice, stream));
			(void)launchDependent(bp::applyRemovedKernel, divUp(nbRemoved, 256), 256, stream, dRemoved.ptr, nbRemoved, live.ptr, flags.ptr);
		}
		if(nbRec)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(dRecs.ptr, hRecs.ptr, size_t(nbRec) * sizeof(bp::UpdateRec), cudaMemcpyHostToDevice, stream));
			(void)launchDependent(bp::applyUpdatesKernel, divUp(nbRec, 256), 256, stream, dRecs.ptr, nbRec, bx.ptr, byz.ptr, groups.ptr, live.ptr, flags.ptr);
		}
		return runFrame(nbRec + nbRemoved, dRecs.ptr, nbRec, true);
	}

	// Everything after the object state is current on the device.
	// updatedRecs: the update records of the created / updated boxes (null: handles
	// [0, nbUpdatedBoxes) were updated from device bounds)
	int runFrame(uint32_t nbTouched, const bp::UpdateRec* updatedRecs, uint32_t nbUpdatedBoxes, bool hostResults)
	{
		// 2. Live boxes sorted by encoded min X: last frame's order without the
		// removed and updated boxes, merged with the created / updated ones sorted.
		const uint32_t nPrevOrder = nOrder;
		const uint32_t* prevOrder = order[orderSide].ptr;
		uint32_t nbS = 0;
		if(nPrevOrder)
		{
			if(keepFlag.reserve(nPrevOrder + 1) || keptPos.reserve(nPrevOrder + 1)) return GBPX_ERR_NOMEM;
			(void)launchDependent(bp::keepFlagKernel, divUp(nPrevOrder, 256), 256, stream, prevOrder, nPrevOrder, live.ptr, flags.ptr, keepFlag.ptr);
			if(compactFlag(keepFlag.ptr, nPrevOrder, 1u, keptPos.ptr)) return GBPX_ERR_NOMEM;
			GBPX_CUDA_TRY(cudaMemcpyAsync(hCounts.ptr, blockCounts.ptr + divUp(nPrevOrder, 256), 4, cudaMemcpyDeviceToHost, stream));
			GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
			nbS = hCounts.ptr[0];
		}
		const uint32_t nbU = nbUpdatedBoxes;
		const uint32_t n = nbS + nbU;
		if(keysA.reserve(nbU + 1) || valsA.reserve(nbU + 1) || keysB.reserve(nbU + 1) || valsB.reserve(nbU + 1) ||
		   hist.reserve(radixSortHistEntries(nbU) + 1) || keptIds.reserve(nbS + 1) || keptKeys.reserve(nbS + 1) ||
		   order[orderSide ^ 1u].reserve(n + 1) || sx.reserve(n + 1) || syz.reserve(n + 1) || sgrp.reserve(n + 1) || supd.reserve(n + 1) ||
		   updPos.reserve(nbU + 1) || sleepPos.reserve(nbS + 1))
			return GBPX_ERR_NOMEM;
		if(nbU) (void)launchDependent(bp::updatedKeysKernel, divUp(nbU, 256), 256, stream, updatedRecs, nbU, bx.ptr, keysA.ptr, valsA.ptr);
		const bool alt = radixSort<uint32_t, true>(keysA.ptr, valsA.ptr, keysB.ptr, valsB.ptr, nbU, 0, 32, hist.ptr, stream);
		const uint32_t* uKeys = alt ? keysB.ptr : keysA.ptr;
		const uint32_t* uIds = alt ? valsB.ptr : valsA.ptr;
		if(nbS)
			(void)launchDependent(bp::gatherKeptKernel, divUp(nbS, 256), 256, stream, prevOrder, keptPos.ptr, nbS, bx.ptr, keptIds.ptr, keptKeys.ptr);
		uint32_t* sortedIds = order[orderSide ^ 1u].ptr;
		if(n)
		{
			(void)launchDependent(bp::mergeOrderKernel, divUp(n, 256), 256, stream, uKeys, uIds, nbU, keptKeys.ptr, keptIds.ptr, nbS, sortedIds,
			                      updPos.ptr, sleepPos.ptr);
			(void)launchDependent(bp::gatherSortedKernel, divUp(n, 256), 256, stream, sortedIds, n, bx.ptr, byz.ptr, groups.ptr, flags.ptr, sx.ptr,
			                      syz.ptr, sgrp.ptr, supd.ptr);
		}
		orderSide ^= 1u;
		nOrder = n;

		// 3. The sweep's lists: sorted positions of the updated boxes (updPos) and of
		// the others (sleepPos), both written by the merge.
		const uint32_t nbUpd = nbU;
		const uint32_t nbSleep = nbS;

		// 4. Sweep.  The found buffer grows and the sweep reruns if it overflowed.
		uint32_t nFound = 0;
		if(found.reserve(1024) || foundAlt.reserve(1024) || longScans.reserve(size_t(nbSleep) + 1)) return GBPX_ERR_NOMEM;
		for(int attempt = 0; attempt < 3; attempt++)
		{
			GBPX_CUDA_TRY(cudaMemsetAsync(counter.ptr, 0, 16, stream));
			const uint32_t capF = uint32_t(std::min<size_t>(found.cap, 0xffffffffu));
			if(nbUpd)
			{
				unsigned long long* longCount = reinterpret_cast<unsigned long long*>(counter.ptr + 2);
				if(sweepTiled)
					(void)launchDependent(bp::sweepUpdatedTiledKernel, std::min<uint32_t>(divUp(nbUpd, bp::UPD_PER_BLOCK), 152u * 64u), 256, stream, 
					    updPos.ptr, nbUpd, n, sx.ptr, syz.ptr, sgrp.ptr, sortedIds, lutLo, lutHi, found.ptr, capF, counter.ptr);
				else
				{
					const uint32_t blocks = std::min<uint32_t>(divUp(uint64_t(nbUpd) * 32, 256), 152u * 64u);
					(void)launchDependent(bp::sweepUpdatedKernel, blocks, 256, stream, updPos.ptr, nbUpd, n, sx.ptr, syz.ptr, sgrp.ptr, sortedIds, lutLo, lutHi,
					                                                  found.ptr, capF, counter.ptr);
				}
				if(nbSleep)
				{
					if(sweepTiled)
						(void)launchDependent(bp::sweepSleepingTiledKernel, std::min<uint32_t>(divUp(nbSleep, bp::SLEEP_PER_BLOCK), 152u * 64u), 256, stream, 
						    sleepPos.ptr, nbSleep, updPos.ptr, nbUpd, sx.ptr, syz.ptr, sgrp.ptr, sortedIds, lutLo, lutHi, found.ptr, capF,
						    counter.ptr, longScans.ptr, longCount);
					else
						(void)launchDependent(bp::sweepSleepingKernel, divUp(nbSleep, 256), 256, stream, sleepPos.ptr, nbSleep, updPos.ptr, nbUpd, sx.ptr, syz.ptr,
						                                                                 sgrp.ptr, sortedIds, lutLo, lutHi, found.ptr, capF,
						                                                                 counter.ptr, longScans.ptr, longCount);
					(void)launchDependent(bp::sweepLongKernel, 152u * 8u, 256, stream, longScans.ptr, reinterpret_cast<const unsigned long long*>(counter.ptr + 2),
					                                                    updPos.ptr, sx.ptr, syz.ptr, sgrp.ptr, sortedIds, lutLo, lutHi, found.ptr,
					                                                    capF, counter.ptr);
				}
			}
			GBPX_CUDA_TRY(cudaMemcpyAsync(hCounts.ptr, counter.ptr, 4, cudaMemcpyDeviceToHost, stream));
			GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
			nFound = hCounts.ptr[0];
			if(nFound <= capF) break;
			if(found.reserve(size_t(nFound) + 1024) || foundAlt.reserve(size_t(nFound) + 1024)) return GBPX_ERR_NOMEM;
			if(attempt == 2) return GBPX_ERR_CAPACITY;
		}

		// 5. Deterministic order: sort the found keys.
		if(hist.reserve(radixSortHistEntries(nFound) + 1)) return GBPX_ERR_NOMEM;
		unsigned long long* F = found.ptr;
		if(nFound > 1)
		{
			// keys are (id0 << 32) | id1 with ids below the capacity: the digits above its bit
			// width in each half are zero and are skipped
			int idBits = 1;
			while(idBits < 32 && (1ull << idBits) < capacity) idBits++;
			uint32_t skip = 0;
			for(int d = 0; d < 8; d++)
				if((d * 8) % 32 >= idBits) skip |= 1u << d;
			const bool a2 = radixSort<unsigned long long, false>(found.ptr, nullptr, foundAlt.ptr, nullptr, nFound, 0, 64, hist.ptr, stream, skip);
			F = a2 ? foundAlt.ptr : found.ptr;
		}

		// 6. Created / lost / next active set; the counts stay on the device until the
		// frame's one synchronisation (fetchResults / updateFromDevice).
		const uint32_t m = std::max(nFound, nPrev) + 1;
		if(cls.reserve(m) || sel.reserve(m) || pos.reserve(m + 1) || created.reserve(m) || lost.reserve(m) || next.reserve(size_t(nFound) + nPrev + 1) ||
		   prev.reserve(1) || frameCounts.reserve(4) || hFrameCounts.reserve(4) ||
		   (hostResults && (hCreated.reserve(size_t(nFound) + 1) || hLost.reserve(size_t(nPrev) + 1))))
			return GBPX_ERR_NOMEM;
		GBPX_CUDA_TRY(cudaMemsetAsync(frameCounts.ptr, 0, 16, stream));
		uint32_t* dCreated = frameCounts.ptr + 0;
		uint32_t* dLost = frameCounts.ptr + 1;
		uint32_t* dKeep = frameCounts.ptr + 2;
		uint32_t* dNext = frameCounts.ptr + 3;
		if(nFound)
		{
			(void)launchDependent(bp::classifyFoundKernel, divUp(nFound, 256), 256, stream, F, nFound, prev.ptr, nPrev, sel.ptr);
			int r2 = scanToDevice(sel.ptr, nFound, pos.ptr, dCreated);
			if(r2) return r2;
			(void)launchDependent(bp::scatterSelectedKernel, divUp(nFound, 256), 256, stream, F, sel.ptr, pos.ptr, nFound, created.ptr);
		}
		DevBuf<unsigned long long>& keepBuf = foundAlt.ptr == F ? found : foundAlt;  // the sort buffer not holding F
		if(keepBuf.reserve(size_t(nPrev) + 1)) return GBPX_ERR_NOMEM;
		unsigned long long* keep = keepBuf.ptr;
		if(nPrev)
		{
			(void)launchDependent(bp::classifyPrevKernel, divUp(nPrev, 256), 256, stream, prev.ptr, nPrev, F, nFound, flags.ptr, cls.ptr);
			(void)launchDependent(bp::flagEqualsKernel, divUp(nPrev, 256), 256, stream, cls.ptr, nPrev, 2u, sel.ptr);
			int r2 = scanToDevice(sel.ptr, nPrev, pos.ptr, dLost);
			if(r2) return r2;
			(void)launchDependent(bp::scatterSelectedKernel, divUp(nPrev, 256), 256, stream, prev.ptr, sel.ptr, pos.ptr, nPrev, lost.ptr);
			(void)launchDependent(bp::flagEqualsKernel, divUp(nPrev, 256), 256, stream, cls.ptr, nPrev, 1u, sel.ptr);
			r2 = scanToDevice(sel.ptr, nPrev, pos.ptr, dKeep);
			if(r2) return r2;
			(void)launchDependent(bp::scatterSelectedKernel, divUp(nPrev, 256), 256, stream, prev.ptr, sel.ptr, pos.ptr, nPrev, keep);
		}
		// the next active set: kept pairs merged with the found ones (sizes bounded by nPrev, nFound)
		if(nPrev + nFound)
			(void)launchDependent(bp::mergeCountedKernel, divUp(nPrev + nFound, 256), 256, stream, keep, dKeep, nPrev, F, nFound, next.ptr, dNext);
		std::swap(prev, next);

		// 7. Results to the host (owned by the broadphase until the next update): the
		// pair lists are written straight into pinned host memory, only as many pairs
		// as the device counts hold (created <= found, lost <= previous active).
		if(hostResults)
		{
			uint2* dHostCreated = nullptr;
			uint2* dHostLost = nullptr;
			GBPX_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&dHostCreated), hCreated.ptr, 0));
			GBPX_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&dHostLost), hLost.ptr, 0));
			if(nFound)
				(void)launchDependent(bp::keysToPairsCountedKernel, divUp(nFound, 256), 256, stream, created.ptr, dCreated, dHostCreated);
			if(nPrev)
				(void)launchDependent(bp::keysToPairsCountedKernel, divUp(nPrev, 256), 256, stream, lost.ptr, dLost, dHostLost);
		}
		GBPX_CUDA_TRY(cudaMemcpyAsync(hFrameCounts.ptr, frameCounts.ptr, 16, cudaMemcpyDeviceToHost, stream));
		if(evEnd) GBPX_CUDA_TRY(cudaEventRecord(evEnd, stream));
		stats[0] = n; stats[1] = nbUpd; stats[2] = nFound;
		(void)nbTouched;
		pending = true;
		return GBPX_OK;
	}

	// Handles [0, n) (already created) take new bounds from device memory and are
	// marked updated; the frame runs at once and its active set stays on the
	// device (activePairs).  The created/lost lists are not fetched.
	int updateFromDevice(const float* dBounds, uint32_t n)
	{
		if(pending || n > capacity) return GBPX_ERR_STATE;
		GBPX_CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, capacity, stream));
		if(n) (void)launchDependent(bp::applyDeviceBoundsKernel, divUp(n, 256), 256, stream, dBounds, n, bx.ptr, byz.ptr, flags.ptr);
		const int rc = runFrame(n, nullptr, n, false);
		if(rc) return rc;
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		finishFrame();
		pending = false;
		return GBPX_OK;
	}

	int fetchResults(const uint2** outCreated, uint32_t* nbCreated, const uint2** outLost, uint32_t* nbLost)
	{
		if(!pending) return GBPX_ERR_STATE;
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		GBPX_CUDA_TRY(cudaGetLastError());
		finishFrame();
		pending = false;
		if(evBegin && evEnd && cudaEventElapsedTime(&lastDeviceMs, evBegin, evEnd) != cudaSuccess) lastDeviceMs = -1.0f;
		*outCreated = hCreated.ptr;
		*nbCreated = nbCreatedOut;
		*outLost = hLost.ptr;
		*nbLost = nbLostOut;
		return GBPX_OK;
	}
};
} // namespace gbpx

using gbpx::BroadPhase;

namespace gbpx
{
namespace bpi
{
int updateFromDevice(void* bp, const float* dBounds, uint32_t n) { return static_cast<BroadPhase*>(bp)->updateFromDevice(dBounds, n); }
const unsigned long long* activePairs(void* bp, uint32_t* count)
{
	BroadPhase* b = static_cast<BroadPhase*>(bp);
	*count = b->nPrev;
	return b->prev.ptr;
}
cudaStream_t stream(void* bp) { return static_cast<BroadPhase*>(bp)->stream; }
} // namespace bpi
} // namespace gbpx

GBPX_API int gbpx_bp_create(int discardStaticVsKinematic, int discardKinematicVsKinematic, void** outBp)
{
	if(!outBp) return GBPX_ERR_INVALID;
	BroadPhase* bp = new BroadPhase;
	const int rc = bp->init(discardStaticVsKinematic != 0, discardKinematicVsKinematic != 0);
	if(rc) { bp->release(); delete bp; return rc; }
	*outBp = bp;
	return GBPX_OK;
}

GBPX_API void gbpx_bp_release(void* bp)
{
	if(!bp) return;
	static_cast<BroadPhase*>(bp)->release();
	delete static_cast<BroadPhase*>(bp);
}

GBPX_API uint32_t gbpx_bp_static_filter_group(void) { return 0u; }
GBPX_API uint32_t gbpx_bp_dynamic_filter_group(uint32_t id) { return ((id + 1u) << 3) | 2u; }
GBPX_API uint32_t gbpx_bp_kinematic_filter_group(uint32_t id) { return ((id + 1u) << 3) | 1u; }

GBPX_API int gbpx_bp_update(void* bp, const uint32_t* created, uint32_t nbCreated, const uint32_t* updated, uint32_t nbUpdated,
                            const uint32_t* removed, uint32_t nbRemoved, const float* bounds, const uint32_t* groups,
                            const float* distances, uint32_t capacity)
{
	gbpx::Zone zone("gbpx::bp::update");
	if(!bp) return GBPX_ERR_INVALID;
	return static_cast<BroadPhase*>(bp)->update(created, nbCreated, updated, nbUpdated, removed, nbRemoved, bounds, groups, distances,
	                                            capacity);
}

GBPX_API int gbpx_bp_fetch_results(void* bp, const uint32_t** created, uint32_t* nbCreated, const uint32_t** lost, uint32_t* nbLost)
{
	gbpx::Zone zone("gbpx::bp::fetchResults");
	if(!bp || !created || !nbCreated || !lost || !nbLost) return GBPX_ERR_INVALID;
	const uint2 *c = nullptr, *l = nullptr;
	const int rc = static_cast<BroadPhase*>(bp)->fetchResults(&c, nbCreated, &l, nbLost);
	*created = reinterpret_cast<const uint32_t*>(c);
	*lost = reinterpret_cast<const uint32_t*>(l);
	return rc;
}

GBPX_API int gbpx_bp_stats(void* bp, uint64_t* out4)
{
	if(!bp || !out4) return GBPX_ERR_INVALID;
	memcpy(out4, static_cast<BroadPhase*>(bp)->stats, sizeof(uint64_t) * 4);
	return GBPX_OK;
}

// Sweep kernels of the following updates: 1 = shared-memory tiled (default),
// 0 = one warp per updated box and one thread per other box.  Same pairs.
GBPX_API int gbpx_bp_set_sweep(void* bp, int tiled)
{
	if(!bp || (tiled != 0 && tiled != 1)) return GBPX_ERR_INVALID;
	static_cast<BroadPhase*>(bp)->sweepTiled = tiled;
	return GBPX_OK;
}

// Timing of the last update + fetchResults: out2[0] = host milliseconds staging
// the user's arrays (the gather of the created and updated boxes), out2[1] =
// device milliseconds from the first upload to the results in host memory.
GBPX_API int gbpx_bp_timing(void* bp, float* out2)
{
	if(!bp || !out2) return GBPX_ERR_INVALID;
	out2[0] = static_cast<BroadPhase*>(bp)->lastHostMs;
	out2[1] = static_cast<BroadPhase*>(bp)->lastDeviceMs;
	return GBPX_OK;
}
