// Stable LSD radix sort (8-bit digits) for 32- and 64-bit keys with optional
// 32-bit values.  Hand-written for sm_103a: per-tile digit histograms, one
// scan over the (digit-major) histogram table, then a stable scatter where
// each warp ranks its keys with __match_any_sync and a per-warp counter row
// in shared memory.
//
// Tiles are 256 threads x 8 keys.  Warp w of a tile owns the contiguous key
// range [w*256, w*256+256) of the tile, which keeps the scatter stable.
#pragma once
#include "common.cuh"

namespace gbpx
{
namespace rs
{
constexpr int THREADS = 256;
constexpr int ITEMS = 8;
constexpr int TILE = THREADS * ITEMS;
constexpr int WARPS = THREADS / 32;
constexpr int WARP_SPAN = 32 * ITEMS;

template <typename K>
__global__ void __launch_bounds__(THREADS) histogramKernel(const K* __restrict__ keys, uint32_t n, int shift, uint32_t numTiles,
                                                           uint32_t* __restrict__ hist)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t h[256];
	h[threadIdx.x] = 0;
	__syncthreads();
	const uint64_t base = uint64_t(blockIdx.x) * TILE;
#pragma unroll
	for(int i = 0; i < ITEMS; i++)
	{
		const uint64_t idx = base + uint64_t(i) * THREADS + threadIdx.x;
		if(idx < n)
		{
			const uint32_t d = uint32_t(keys[idx] >> shift) & 0xffu;
			atomicAdd(&h[d], 1u);
		}
	}
	__syncthreads();
	hist[uint64_t(threadIdx.x) * numTiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of the 4096-entry chunk of data starting at `start` by a block
// of 1024 threads (4 entries each), offset by `carry`; returns, in every thread,
// carry plus the chunk's sum.  warpSums: 32 shared words.
__device__ __forceinline__ uint32_t scanChunk(uint32_t* __restrict__ data, uint32_t count, uint32_t start, uint32_t carry, uint32_t* warpSums)
{
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t v[4];
	uint32_t local = 0;
	const uint32_t b = start + threadIdx.x * 4;
#pragma unroll
	for(int k = 0; k < 4; k++)
	{
		v[k] = (b + k < count) ? data[b + k] : 0u;
		local += v[k];
	}
	uint32_t incl = local;
#pragma unroll
	for(int o = 1; o < 32; o <<= 1)
	{
		const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= uint32_t(o)) incl += t;
	}
	if(lane == 31) warpSums[warp] = incl;
	__syncthreads();
	if(warp == 0)
	{
		uint32_t ws = warpSums[lane];
		uint32_t wi = ws;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1)
		{
			const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
			if(lane >= uint32_t(o)) wi += t;
		}
		warpSums[lane] = wi - ws;
		if(lane == 31) warpSums[32] = wi;   // the chunk's total
	}
	__syncthreads();
	uint32_t run = carry + warpSums[warp] + incl - local;
#pragma unroll
	for(int k = 0; k < 4; k++)
	{
		if(b + k < count) data[b + k] = run;
		run += v[k];
	}
	const uint32_t total = carry + warpSums[32];
	__syncthreads();
	return total;
}

constexpr uint32_t SCAN_CHUNK = 1024 * 4;

// Exclusive scan of `count` u32 values in place by one block of 1024 threads.
static __global__ void __launch_bounds__(1024) scanKernel(uint32_t* __restrict__ data, uint32_t count)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpSums[33];
	uint32_t carry = 0;
	for(uint32_t start = 0; start < count; start += SCAN_CHUNK) carry = scanChunk(data, count, start, carry, warpSums);
}

// Sum of each SCAN_CHUNK-entry chunk of data: chunk b -> sums[b].
static __global__ void __launch_bounds__(1024) chunkSumKernel(const uint32_t* __restrict__ data, uint32_t count, uint32_t* __restrict__ sums)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpSums[32];
	const uint32_t b = blockIdx.x * SCAN_CHUNK + threadIdx.x * 4;
	uint32_t local = 0;
#pragma unroll
	for(int k = 0; k < 4; k++) local += (b + k < count) ? data[b + k] : 0u;
	for(int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
	if((threadIdx.x & 31) == 0) warpSums[threadIdx.x >> 5] = local;
	__syncthreads();
	if(threadIdx.x < 32)
	{
		uint32_t v = warpSums[threadIdx.x];
		for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
		if(threadIdx.x == 0) sums[blockIdx.x] = v;
	}
}

// Exclusive scan of chunk b of data, offset by offsets[b] (the exclusive scan of the chunk sums).
static __global__ void __launch_bounds__(1024) chunkScanKernel(uint32_t* __restrict__ data, uint32_t count, const uint32_t* __restrict__ offsets)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpSums[33];
	scanChunk(data, count, blockIdx.x * SCAN_CHUNK, offsets[blockIdx.x], warpSums);
}

// Entries of the scratch scanAny needs for `count` values.
static inline uint32_t scanScratchEntries(uint32_t count) { return uint32_t((count + SCAN_CHUNK - 1) / SCAN_CHUNK + 1); }

// Exclusive scan of data[0..count) in place: one block for short arrays, else
// chunk sums, a scan of the sums and a scan of every chunk in parallel.
static inline void scanAny(uint32_t* data, uint32_t count, uint32_t* scratch, cudaStream_t s)
{
	if(count <= 4 * SCAN_CHUNK)
	{
		(void)launchDependent(scanKernel, 1, 1024, s, data, count);
		return;
	}
	const uint32_t chunks = (count + SCAN_CHUNK - 1) / SCAN_CHUNK;
	(void)launchDependent(chunkSumKernel, chunks, 1024, s, data, count, scratch);
	(void)launchDependent(scanKernel, 1, 1024, s, scratch, chunks);
	(void)launchDependent(chunkScanKernel, chunks, 1024, s, data, count, scratch);
}

template <typename K, bool HAS_VAL>
__global__ void __launch_bounds__(THREADS) scatterKernel(const K* __restrict__ keysIn, const uint32_t* __restrict__ valsIn,
                                                         K* __restrict__ keysOut, uint32_t* __restrict__ valsOut, uint32_t n,
                                                         int shift, uint32_t numTiles, const uint32_t* __restrict__ offsets)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t cnt[WARPS][256];
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for(int d = threadIdx.x; d < WARPS * 256; d += THREADS) (&cnt[0][0])[d] = 0;
	__syncthreads();

	const uint64_t base = uint64_t(blockIdx.x) * TILE + uint64_t(warp) * WARP_SPAN;
	K key[ITEMS];
	uint32_t val[ITEMS];
	uint32_t rank[ITEMS];
	const uint32_t lt = laneMaskLt();
#pragma unroll
	for(int i = 0; i < ITEMS; i++)
	{
		const uint64_t idx = base + uint64_t(i) * 32 + lane;
		const bool valid = idx < n;
		key[i] = valid ? keysIn[idx] : K(0);
		if(HAS_VAL) val[i] = valid ? valsIn[idx] : 0u;
		const uint32_t d = valid ? (uint32_t(key[i] >> shift) & 0xffu) : 0x100u;
		const uint32_t peers = __match_any_sync(0xffffffffu, d);
		uint32_t c = 0;
		if(valid) c = cnt[warp][d];
		__syncwarp();
		rank[i] = c + __popc(peers & lt);
		const bool leader = (peers & lt) == 0;
		if(valid && leader) cnt[warp][d] = c + __popc(peers);
		__syncwarp();
	}
	__syncthreads();
	{
		const uint32_t d = threadIdx.x;  // THREADS == 256 digits
		uint32_t run = offsets[uint64_t(d) * numTiles + blockIdx.x];
#pragma unroll
		for(int w = 0; w < WARPS; w++)
		{
			const uint32_t t = cnt[w][d];
			cnt[w][d] = run;
			run += t;
		}
	}
	__syncthreads();
#pragma unroll
	for(int i = 0; i < ITEMS; i++)
	{
		const uint64_t idx = base + uint64_t(i) * 32 + lane;
		if(idx < n)
		{
			const uint32_t d = uint32_t(key[i] >> shift) & 0xffu;
			const uint32_t dst = cnt[warp][d] + rank[i];
			keysOut[dst] = key[i];
			if(HAS_VAL) valsOut[dst] = val[i];
		}
	}
}
} // namespace rs

// Scratch needed by radixSort for n keys (histogram table and the scan's chunk
// sums, u32 entries).
static inline size_t radixSortHistEntries(uint32_t n)
{
	const size_t table = size_t(256) * (divUp(n ? n : 1, rs::TILE));
	return table + rs::scanScratchEntries(uint32_t(table));
}

// Sorts keys[0..n) (and vals) on bits [beginBit, endBit).  Ping-pongs between
// (keys, vals) and (keysAlt, valsAlt); returns true if the result ended in the
// Alt buffers.  skipDigits: bit d set when digit d (bits 8d .. 8d+7) is the same
// in every key, so its pass (a stable sort on a constant) is skipped.
template <typename K, bool HAS_VAL>
static bool radixSort(K* keys, uint32_t* vals, K* keysAlt, uint32_t* valsAlt, uint32_t n, int beginBit, int endBit,
                      uint32_t* hist, cudaStream_t s, uint32_t skipDigits = 0)
{
	if(n <= 1) return false;
	const uint32_t numTiles = divUp(n, rs::TILE);
	bool inAlt = false;
	for(int shift = beginBit; shift < endBit; shift += 8)
	{
		if((skipDigits >> (shift / 8)) & 1u) continue;
		const K* kin = inAlt ? keysAlt : keys;
		const uint32_t* vin = inAlt ? valsAlt : vals;
		K* kout = inAlt ? keys : keysAlt;
		uint32_t* vout = inAlt ? vals : valsAlt;
		(void)launchDependent(rs::histogramKernel<K>, numTiles, rs::THREADS, s, kin, n, shift, numTiles, hist);
		rs::scanAny(hist, 256u * numTiles, hist + 256u * numTiles, s);
		(void)launchDependent(rs::scatterKernel<K, HAS_VAL>, numTiles, rs::THREADS, s, kin, vin, kout, vout, n, shift, numTiles, hist);
		inAlt = !inAlt;
	}
	return inAlt;
}
} // namespace gbpx
