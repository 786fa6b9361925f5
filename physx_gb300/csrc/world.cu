// Batched multi-scene rigid-body step for the GB300.
//
// Thousands of independent scenes advance together, one CUDA graph per step.
// The scene stages pull scenes from a work table sorted by decreasing size
// (largest first, so the tail is short); scenes of up to `largeBodies` solver
// bodies run one warp per scene, larger ones one block of 8 warps per scene
// (on a side stream, concurrently):
//   1. bounds + broadphase: AABBs, bitonic sort by encoded min X, sweep with the
//      reference ABP's closed-interval test (X as encodeFloat keys, Y/Z as
//      floats), pairs ordered by (id0, id1), statics after the dynamic bodies,
//      each pair queued under its pair kind;
//   2. narrowphase: one kernel per pair kind over every scene's pairs, a thread
//      per pair, PxGenerateContacts semantics (contacts.cuh);
//   3. batching: solver bodies and the PxBatchConstraintsTGS partition rule;
//   4. row preparation: a thread per constraint;
//   5. solve: position iterations with per-substep integration and the velocity
//      iteration, partition by partition (constraints of one partition touch
//      disjoint bodies), then PxIntegrateSolverBodiesTGS and write-back; by
//      default the resident solve, which bulk-copies each scene's rows and
//      velocities into shared memory once and runs every iteration there.
// All scene state stays resident in HBM.
//
// The step is the reference immediate-mode snippet's frame (physx/snippets/
// snippetimmediatemode/SnippetImmediateMode.cpp:473 stepPhysics): bounds
// inflated by a margin, ABP pairs, PxGenerateContacts, PxConstructSolverBodiesTGS,
// PxBatchConstraintsTGS, PxCreateContactConstraintsTGS, PxSolveConstraintsTGS,
// PxIntegrateSolverBodiesTGS; in persistent mode (the snippet's default) each
// pair keeps its PCM manifold and friction patches between steps
// (SnippetImmediateMode.cpp:657-676, 941-978), double-buffered per scene.
#include "common.cuh"
#include "contacts.cuh"
#include "solver.cuh"
#include "step_common.cuh"
#include <vector>
#include <algorithm>
#include <numeric>
#include <chrono>
#include <deque>
#include <random>
#include <map>
#include <string>

namespace gbpx
{
namespace world
{
constexpr uint32_t MAX_PARTITIONS = 128;
enum : uint32_t { ST_PAIR_OVERFLOW = 1, ST_PARTITION_OVERFLOW = 2, ST_STAGE_TIMEOUT = 4 };

// Resident solve (solveResidentKernel): one block of RES_WARPS warps per SM
// with the whole opt-in shared memory as its workspace.  Each scene's packed
// rows and body velocities are copied on chip once and stay there for all
// iterations.  Scenes are filed by on-chip footprint into RES_LEVELS levels:
// at level L the block works as 2^L groups of RES_WARPS >> L warps, each group
// solving one scene at a time in 1/2^L of the workspace.
constexpr uint32_t RES_WARPS = 16;
constexpr uint32_t RES_LEVELS = 5;
static_assert((RES_WARPS >> (RES_LEVELS - 1)) >= 1 && RES_WARPS <= 16, "levels down to one warp; named barriers 1..RES_WARPS-1");
constexpr uint32_t RES_HEADER = MAX_PARTITIONS * 4;   // partition ends at the start of a group's slice
// work counters of the persistent stage kernels (scenes or entries taken)
enum : uint32_t { WC_BP = 0, WC_BATCH = 1, WC_SOLVE = 2, WC_PREP = 3, WC_BP_BIG = 4, WC_BATCH_BIG = 5, WC_SOLVE_BIG = 6 };
// work counters (after the per-kind pair counts and path counts): scenes filed
// per level, then scenes taken per level
constexpr uint32_t WC_RES_COUNT = 8 + 9 + 4;
constexpr uint32_t WC_RES_NEXT = WC_RES_COUNT + RES_LEVELS;
// the row preparation's queue classes (constraints with the same path, contact
// count and count of last step's friction patches): entries per class, then
// entries placed per class
constexpr uint32_t PREP_CLASSES = 32;
constexpr uint32_t WC_PREP_CLASS = WC_RES_NEXT + RES_LEVELS;
constexpr uint32_t WC_PREP_PLACED = WC_PREP_CLASS + PREP_CLASSES;
// pairs taken per pair kind by the narrowphase kernels' warps
constexpr uint32_t WC_NP_TAKEN = WC_PREP_PLACED + PREP_CLASSES;
constexpr uint32_t NB_WORK_COUNTERS = WC_NP_TAKEN + 9;
// StepParams::solveVariant selecting the resident solve (0-7 are staging
// variants of the warp-per-scene solve)
constexpr uint32_t RESIDENT_VARIANT = 8;

__host__ __device__ __forceinline__ uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }
// On-chip bytes of a scene in the resident solve: partition ends, 16-bit row
// offsets (16-byte units), lin / ang / dLin / dAng of every solver body, rows.
__host__ __device__ __forceinline__ uint32_t residentBytes(uint32_t nc, uint32_t nTot, uint32_t rowChunks)
{
	return RES_HEADER + align16(2 * nc) + align16(48 * nTot) + 16 * rowChunks;
}
// Streamed rows (a scene whose rows do not fit its slice): each iteration's
// rows arrive chunk by chunk (consecutive constraints of one partition, at
// most a ring slot) in a two-slot ring, the next chunk's bulk copies running
// while the current one is solved; the solve writes each constraint's
// impulses back to its record in HBM, where the next iteration's copy reads
// them.  Footprint: partition ends, row offsets, velocities, the chunk table
// and two slots of at least RES_MIN_SLOT bytes.
constexpr uint32_t RES_MAX_CHUNKS = 256;   // chunks of one iteration
constexpr uint32_t RES_TABLE = (RES_MAX_CHUNKS + 1 + MAX_PARTITIONS + 1 + 2) * 4;   // chunk starts, first chunk per partition, total
constexpr uint32_t RES_MIN_SLOT = 16384;
constexpr uint32_t RES_RECORD_UNITS = 56;  // 16-byte units of the largest constraint record
__host__ __device__ __forceinline__ uint32_t residentStreamBytes(uint32_t nc, uint32_t nTot)
{
	return RES_HEADER + align16(2 * nc) + align16(48 * nTot) + align16(RES_TABLE) + 2 * RES_MIN_SLOT;
}
// Smallest slice (deepest level) that holds `need` bytes; level 0 also takes
// scenes too large for any slice (their rows stay in HBM).
__host__ __device__ __forceinline__ uint32_t residentLevel(uint32_t need, uint32_t resBytes)
{
	uint32_t L = 0;
	while(L + 1 < RES_LEVELS && need <= (resBytes >> (L + 1))) L++;
	return L;
}

struct SceneDesc
{
	uint32_t bodyStart, nbBodies;      // dynamic bodies [bodyStart, bodyStart + nbBodies)
	uint32_t staticStart, nbStatics;   // static shapes
	uint32_t solverStart;              // solver bodies [solverStart, + nbBodies + nbStatics)
	uint32_t keyStart, keyCap;         // sort keys (power of two >= nbBodies)
	uint32_t pairStart, pairCap;       // pair / contact / constraint slots (power of two)
};

struct WorldDev
{
	const SceneDesc* scenes;
	const uint32_t* workOrder;  // scenes to step, largest first
	const uint32_t* nbActive;   // entries of workOrder to step (device word, so a captured step serves any scene set)
	uint32_t* workCounter;
	tgs::RigidBody* bodies;
	const int* types;
	const float4* geoms;
	const float* friction;
	const float* staticPose;   // 7 floats
	const int* staticTypes;
	const float4* staticGeoms;
	float* aabb;               // 6 floats per dynamic body
	unsigned long long* keys;
	uint32_t* pairs;
	uint32_t* pairCount;
	float4* contacts;          // 8 float4 per pair slot
	uint32_t* contactCount;
	uint32_t* ordered;         // per pair slot: constraint order (pair index)
	uint32_t* consList;        // per pair slot: pairs with contacts
	uint32_t* tag;             // per pair slot: (round << 8) | partition, 0xffff for static constraints
	tgs::ConstraintRecord* recs;
	tgs::BodyVel* vel;
	tgs::BodyTx* tx;
	tgs::BodyData* data;
	Tr* pose;
	uint32_t* progress;        // per solver body
	uint32_t* maxNormal;
	uint32_t* maxStatic;
	uint32_t* staticProgress;
	uint32_t* partEnds;        // MAX_PARTITIONS per scene
	uint32_t* status;
	uint32_t* typeCount;       // pairs queued per pair kind (NB_KINDS)
	uint32_t* pathCount;       // capsule-box, box-box: pairs ordered to the front (refresh) / back (full path)
	uint32_t* typeQueueSorted; // capsule-box, box-box queues ordered by contact-generation path (persistent mode)
	uint32_t* typeQueue;       // NB_KINDS queues of pair slots, queueCap entries each
	uint32_t queueCap;
	const uint32_t* slotScene; // owning scene of every pair slot
	uint32_t* nbConstraints;   // per scene: constraints (pairs with contacts) of this step
	uint32_t* nbPartitions;    // per scene: partitions, 0 when batching overflowed
	uint32_t* prepQueue;       // constraint slots of all scenes, for the row-preparation kernel
	uint8_t* prepClass;        // class of each prepQueue entry
	uint32_t* prepQueueSorted; // prepQueue grouped by class (what prepKernel reads)
	uint8_t* recChunks;        // per constraint slot: 16-byte chunks its packed rows occupy
	// Persistent pair state (the reference snippet's persistent mode): per pair
	// slot a contact manifold and the friction patches its constraint left, in
	// two buffers; sceneParity[scene] names the one holding the last step's.
	uint32_t* pairsPrev;       // per pair slot: last step's pair keys
	uint32_t* pairCountPrev;   // per scene
	uint32_t* prevSlot;        // per pair slot: the pair's index in last step's list, or NO_PREV
	uint32_t* sceneParity;     // per scene
	np::ManifoldRecord* manifolds[2];
	tgs::FrictionState* frictionState[2];
	// Resident solve: per scene, constraints prepared and their row chunks
	// (count << 32 | chunks); per footprint level, the scenes to solve.
	unsigned long long* sceneAcc;
	uint32_t* resList;         // RES_LEVELS lists of resCap scene ids
	uint32_t resCap;
};
__device__ __forceinline__ void residentAppend(const WorldDev& w, uint32_t sid, uint32_t level)
{
	const uint32_t i = atomicAdd(&w.workCounter[WC_RES_COUNT + level], 1u);
	w.resList[size_t(level) * w.resCap + i] = sid;
}

// A group of G warps working on one scene: G = 1 is one warp (several scenes
// per block), G > 1 is the whole block (one scene per block, for large scenes).
template <uint32_t G>
struct Grp
{
	static constexpr uint32_t NT = 32 * G;
	__device__ static __forceinline__ uint32_t tid() { return G == 1 ? (threadIdx.x & 31) : threadIdx.x; }
	__device__ static __forceinline__ uint32_t warp() { return G == 1 ? 0u : (threadIdx.x >> 5); }
	__device__ static __forceinline__ void sync()
	{
		if constexpr(G == 1) __syncwarp();
		else __syncthreads();
	}
	// value of thread 0, to every thread of the group (slot: shared scratch word)
	__device__ static __forceinline__ uint32_t bcast(uint32_t v, volatile uint32_t* slot)
	{
		if constexpr(G == 1) return __shfl_sync(0xffffffffu, v, 0);
		else
		{
			if(threadIdx.x == 0) *slot = v;
			__syncthreads();
			const uint32_t r = *slot;
			__syncthreads();
			return r;
		}
	}
};

template <uint32_t G, typename K>
__device__ __forceinline__ void groupBitonicSort(K* keys, uint32_t n)
{
	for(uint32_t k = 2; k <= n; k <<= 1)
	{
		for(uint32_t j = k >> 1; j > 0; j >>= 1)
		{
			for(uint32_t i = Grp<G>::tid(); i < n; i += Grp<G>::NT)
			{
				const uint32_t ixj = i ^ j;
				if(ixj > i)
				{
					const K a = keys[i], b = keys[ixj];
					const bool up = (i & k) == 0;
					if(up ? (a > b) : (a < b)) { keys[i] = b; keys[ixj] = a; }
				}
			}
			Grp<G>::sync();
		}
	}
}

// Exclusive prefix sum of v[0..n) by one group (each thread scans a run of
// entries); scratch: G shared words (unused for G = 1).
template <uint32_t G>
__device__ __forceinline__ void groupExclusiveScan(uint32_t* v, uint32_t n, uint32_t* scratch)
{
	constexpr uint32_t NT = Grp<G>::NT;
	const uint32_t tid = Grp<G>::tid(), lane = threadIdx.x & 31;
	const uint32_t per = (n + NT - 1) / NT;
	const uint32_t b0 = min(tid * per, n), b1 = min(b0 + per, n);
	uint32_t sum = 0;
	for(uint32_t k = b0; k < b1; k++) sum += v[k];
	uint32_t incl = sum;
	for(int o = 1; o < 32; o <<= 1)
	{
		const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= uint32_t(o)) incl += t;
	}
	if constexpr(G > 1)
	{
		const uint32_t warp = Grp<G>::warp();
		if(lane == 31) scratch[warp] = incl;
		__syncthreads();
		uint32_t off = 0;
		for(uint32_t q = 0; q < warp; q++) off += scratch[q];
		incl += off;
	}
	uint32_t run = incl - sum;
	for(uint32_t k = b0; k < b1; k++)
	{
		const uint32_t c = v[k];
		v[k] = run;
		run += c;
	}
	Grp<G>::sync();
}

// Shared-memory workspace of the broadphase of one scene: scenes whose sort
// keys fit (CAP) sort and sweep entirely on chip; larger scenes use the same
// code on their global scratch arrays.  Warp groups use BP_SMEM_BODIES, block
// groups (large scenes) BIG_BP_BODIES.
constexpr uint32_t BP_SMEM_BODIES = 512;
constexpr uint32_t BIG_BP_BODIES = 4096;
constexpr uint32_t STAGE_WARPS = 4;   // warps (scenes in flight) per block of the warp-per-scene kernels
constexpr uint32_t BIG_WARPS = 8;     // warps per block (one scene) of the large-scene kernels
template <uint32_t CAP>
struct BpSmemT
{
	unsigned long long keys[CAP];   // (encoded min X << 32) | body
	uint32_t maxX[CAP];             // encoded max X
	float minY[CAP], minZ[CAP], maxY[CAP], maxZ[CAP];
	uint32_t cnt[CAP];              // pairs per lower body id, then bucket offsets
	uint32_t found, bc;
	uint32_t scan[32];
};
using BpSmem = BpSmemT<BP_SMEM_BODIES>;
using BpSmemBig = BpSmemT<BIG_BP_BODIES>;

// Bounds, ABP-equivalent overlap search and the pair list of one scene, sorted
// by (id0, id1) with statics numbered after the dynamic bodies.
// The sweep follows ABP's semantics: boxes sorted by encoded min X, X
// overlap on encoded keys, Y/Z as closed float intervals.  Found pairs are
// counted per lower id, scattered into their buckets and each bucket sorted by
// the upper id, which yields the same order as sorting the whole list.
template <uint32_t G, uint32_t CAP>
__device__ __forceinline__ void sceneBroadphase(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp, BpSmemT<CAP>& sm)
{
	constexpr uint32_t NT = Grp<G>::NT;
	const uint32_t tid = Grp<G>::tid(), lane = threadIdx.x & 31;
	const uint32_t n = sc.nbBodies, m = sc.nbStatics;
	const bool onChip = sc.keyCap <= CAP;
	unsigned long long* keys = onChip ? sm.keys : w.keys + sc.keyStart;
	float* ga = w.aabb + 6 * size_t(sc.bodyStart);
	uint32_t* maxX = onChip ? sm.maxX : reinterpret_cast<uint32_t*>(ga);
	float* minY = onChip ? sm.minY : ga + n;
	float* minZ = onChip ? sm.minZ : ga + 2 * size_t(n);
	float* maxY = onChip ? sm.maxY : ga + 3 * size_t(n);
	float* maxZ = onChip ? sm.maxZ : ga + 4 * size_t(n);
	uint32_t* cnt = onChip ? sm.cnt : w.progress + sc.solverStart;
	const float mg = sp.boundsMargin;
	if(sp.persistent)
	{
		// last step's pair list, for matching this step's pairs to their state
		const uint32_t prevCount = w.pairCount[sid];
		for(uint32_t t = tid; t < prevCount; t += NT) w.pairsPrev[sc.pairStart + t] = w.pairs[sc.pairStart + t];
		if(tid == 0) w.pairCountPrev[sid] = prevCount;
	}
	for(uint32_t i = tid; i < sc.keyCap; i += NT)
	{
		if(i < n)
		{
			const tgs::RigidBody& rb = w.bodies[sc.bodyStart + i];
			Tr pose;
			pose.q.x = rb.q[0]; pose.q.y = rb.q[1]; pose.q.z = rb.q[2]; pose.q.w = rb.q[3];
			pose.p = v3(rb.p[0], rb.p[1], rb.p[2]);
			V3 mn, mx;
			shapeBounds(w.types[sc.bodyStart + i], w.geoms[sc.bodyStart + i], pose, mn, mx);
			const float x0 = mn.x - mg;
			maxX[i] = encodeFloatBits(__float_as_uint(mx.x + mg));
			minY[i] = mn.y - mg; minZ[i] = mn.z - mg;
			maxY[i] = mx.y + mg; maxZ[i] = mx.z + mg;
			cnt[i] = 0;
			keys[i] = (static_cast<unsigned long long>(encodeFloatBits(__float_as_uint(x0))) << 32) | i;
		}
		else
			keys[i] = ~0ull;
	}
	if(tid == 0) sm.found = 0;
	Grp<G>::sync();
	groupBitonicSort<G>(keys, sc.keyCap);
	uint32_t* scratch = w.ordered + sc.pairStart;   // unsorted pairs (the slot array is free until the solve)
	uint32_t local = 0;   // thread-private overflow flag
	for(uint32_t p = tid; p < n; p += NT)
	{
		const unsigned long long kp = keys[p];
		const uint32_t i = uint32_t(kp);
		const uint32_t amaxx = maxX[i];
		const float a1 = minY[i], a2 = minZ[i], a4 = maxY[i], a5 = maxZ[i];
		for(uint32_t q = p + 1; q < n; q++)
		{
			const unsigned long long kq = keys[q];
			if(uint32_t(kq >> 32) > amaxx) break;
			const uint32_t j = uint32_t(kq);
			if(!(maxY[j] < a1 || a4 < minY[j] || maxZ[j] < a2 || a5 < minZ[j]))
			{
				const uint32_t lo = i < j ? i : j, hi = i < j ? j : i;
				const uint32_t slot = atomicAdd(&sm.found, 1u);
				if(slot < sc.pairCap) { scratch[slot] = (lo << 16) | hi; atomicAdd(&cnt[lo], 1u); } else local = 1;
			}
		}
		if(m)
		{
			const uint32_t aminx = uint32_t(kp >> 32);
			for(uint32_t s = 0; s < m; s++)
			{
				V3 mn, mx;
				const Tr sp7 = loadStaticPose(w.staticPose + 7 * size_t(sc.staticStart + s));
				shapeBounds(w.staticTypes[sc.staticStart + s], w.staticGeoms[sc.staticStart + s], sp7, mn, mx);
				const uint32_t bminx = encodeFloatBits(__float_as_uint(mn.x - mg)), bmaxx = encodeFloatBits(__float_as_uint(mx.x + mg));
				if(bminx > amaxx || aminx > bmaxx) continue;
				if((mx.y + mg) < a1 || a4 < (mn.y - mg) || (mx.z + mg) < a2 || a5 < (mn.z - mg)) continue;
				const uint32_t slot = atomicAdd(&sm.found, 1u);
				if(slot < sc.pairCap) { scratch[slot] = (i << 16) | (n + s); atomicAdd(&cnt[i], 1u); } else local = 1;
			}
		}
	}
	Grp<G>::sync();
	if(local) atomicOr(&w.status[sid], ST_PAIR_OVERFLOW);
	const uint32_t count = min(sm.found, sc.pairCap);
	// bucket by lower id, then sort each bucket by upper id
	groupExclusiveScan<G>(cnt, n, sm.scan);
	uint32_t* pairs = w.pairs + sc.pairStart;
	for(uint32_t t = tid; t < count; t += NT)
	{
		const uint32_t key = scratch[t];
		pairs[atomicAdd(&cnt[key >> 16], 1u)] = key;
	}
	Grp<G>::sync();
	for(uint32_t lo = tid; lo < n; lo += NT)
	{
		const uint32_t b0 = lo ? cnt[lo - 1] : 0, b1 = cnt[lo];
		for(uint32_t x = b0 + 1; x < b1; x++)
		{
			const uint32_t v = pairs[x];
			uint32_t y = x;
			while(y > b0 && pairs[y - 1] > v) { pairs[y] = pairs[y - 1]; y--; }
			pairs[y] = v;
		}
	}
	if(tid == 0) w.pairCount[sid] = count;
	Grp<G>::sync();
	// queue every pair slot under its pair kind (one atomic per kind per 32 pairs)
	for(uint32_t base = Grp<G>::warp() * 32; base < count; base += NT)
	{
		const uint32_t k = base + lane;
		const bool valid = k < count;
		uint32_t kind = NB_KINDS + 1;
		if(valid)
		{
			const uint32_t key = pairs[k];
			const uint32_t i = key >> 16, j = key & 0xffffu;
			const int ti = w.types[sc.bodyStart + i];
			const int tj = j < n ? w.types[sc.bodyStart + j] : w.staticTypes[sc.staticStart + (j - n)];
			kind = kindOf(ti, tj);
			if(kind == NB_KINDS) w.contactCount[sc.pairStart + k] = 0;
		}
		const uint32_t peers = __match_any_sync(0xffffffffu, kind);
		const uint32_t leader = __ffs(peers) - 1;
		uint32_t qbase = 0;
		if(kind < NB_KINDS && lane == leader) qbase = atomicAdd(&w.typeCount[kind], uint32_t(__popc(peers)));
		qbase = __shfl_sync(0xffffffffu, qbase, leader);
		if(kind < NB_KINDS) w.typeQueue[size_t(kind) * w.queueCap + qbase + __popc(peers & laneMaskLt())] = sc.pairStart + k;
	}
}

__device__ __forceinline__ void pairShape(const WorldDev& w, const SceneDesc& sc, uint32_t id, int& type, float g[4], Tr& pose)
{
	if(id < sc.nbBodies)
	{
		const uint32_t b = sc.bodyStart + id;
		type = w.types[b];
		const float4 gg = w.geoms[b];
		g[0] = gg.x; g[1] = gg.y; g[2] = gg.z; g[3] = gg.w;
		const tgs::RigidBody& rb = w.bodies[b];
		pose.q.x = rb.q[0]; pose.q.y = rb.q[1]; pose.q.z = rb.q[2]; pose.q.w = rb.q[3];
		pose.p = v3(rb.p[0], rb.p[1], rb.p[2]);
	}
	else
	{
		const uint32_t s = sc.staticStart + (id - sc.nbBodies);
		type = w.staticTypes[s];
		const float4 gg = w.staticGeoms[s];
		g[0] = gg.x; g[1] = gg.y; g[2] = gg.z; g[3] = gg.w;
		pose = loadStaticPose(w.staticPose + 7 * size_t(s));
	}
}

// Persistent mode: the capsule-box and box-box queues reordered so that pairs
// whose manifold only refreshes come first and pairs that take the full path
// (GJK/EPA, SAT and clipping) last; each warp then runs one path.  Only the
// order of the slots changes: every pair's result is written to its own slot.
__device__ __forceinline__ uint32_t prevSlotOf(const WorldDev& w, const SceneDesc& sc, uint32_t sid, uint32_t key)
{
	uint32_t lo = 0, hi = w.pairCountPrev[sid];
	const uint32_t* pk = w.pairsPrev + sc.pairStart;
	while(lo < hi)
	{
		const uint32_t mid = (lo + hi) >> 1;
		if(pk[mid] < key) lo = mid + 1;
		else hi = mid;
	}
	return lo < w.pairCountPrev[sid] && pk[lo] == key ? lo : NO_PREV;
}

__global__ void __launch_bounds__(128) orderByPathKernel(WorldDev w, StepParams sp)
{
	const uint32_t c7 = w.typeCount[7], c8 = w.typeCount[8];
	const uint32_t lane = threadIdx.x & 31;
	for(uint32_t base = blockIdx.x * blockDim.x; base < c7 + c8; base += gridDim.x * blockDim.x)
	{
		const uint32_t q = base + threadIdx.x;
		const bool valid = q < c7 + c8;
		const uint32_t k = valid && q >= c7 ? 1u : 0u;   // 0 capsule-box, 1 box-box
		bool full = true;
		uint32_t slot = 0;
		if(valid)
		{
			slot = w.typeQueue[size_t(7 + k) * w.queueCap + (k ? q - c7 : q)];
			const uint32_t sid = w.slotScene[slot];
			const SceneDesc sc = w.scenes[sid];
			const uint32_t key = w.pairs[slot];
			int ta, tb;
			float ga[4], gb[4];
			Tr pa, pb;
			pairShape(w, sc, key >> 16, ta, ga, pa);
			pairShape(w, sc, key & 0xffffu, tb, gb, pb);
			const uint32_t prev = prevSlotOf(w, sc, sid, key);
			np::Manifold m;
			if(prev != NO_PREV) np::loadManifold(w.manifolds[w.sceneParity[sid]][sc.pairStart + prev], m);
			if(k) full = np::boxBoxFullPath(v3(ga[0], ga[1], ga[2]), v3(gb[0], gb[1], gb[2]), pa, pb, sp.toleranceLength, m);
			else if(ta == 2) full = np::capsuleBoxFullPath(ga[0], v3(gb[0], gb[1], gb[2]), pa, pb, sp.toleranceLength, m);
			else full = np::capsuleBoxFullPath(gb[0], v3(ga[0], ga[1], ga[2]), pb, pa, sp.toleranceLength, m);
		}
		// warp-aggregated appends per (kind, path): refresh from the front, full from the back
		for(uint32_t g = 0; g < 4; g++)
		{
			const bool mine = valid && (k * 2 + (full ? 1u : 0u)) == g;
			const uint32_t peers = __ballot_sync(0xffffffffu, mine);
			if(!peers) continue;
			const uint32_t leader = __ffs(peers) - 1;
			uint32_t b = 0;
			if(lane == leader) b = atomicAdd(&w.pathCount[g], uint32_t(__popc(peers)));
			b = __shfl_sync(0xffffffffu, b, leader);
			if(mine)
			{
				const uint32_t r = b + __popc(peers & laneMaskLt());
				const uint32_t count = (g >> 1) ? c8 : c7;
				w.typeQueueSorted[size_t(g >> 1) * w.queueCap + ((g & 1) ? count - 1 - r : r)] = slot;
			}
		}
	}
}

// Narrowphase of one pair kind over every scene: a thread per queued pair slot,
// so each warp runs one contact generator on uniform work.
template <int TA, int TB>
__global__ void __launch_bounds__(128, (TA == 3 && TB == 3) ? 4 : 5) narrowphaseKernel(WorldDev w, StepParams sp)
{
	constexpr uint32_t KIND = TA == 0 ? uint32_t(TB) : (TA == 1 ? uint32_t(TB + 2) : (TA == 2 ? uint32_t(TB + 4) : 8u));
	const uint32_t count = w.typeCount[KIND];
	const bool sorted = (KIND == 7 || KIND == 8) && sp.persistent;
	const uint32_t* queue = sorted ? w.typeQueueSorted + size_t(KIND - 7) * w.queueCap : w.typeQueue + size_t(KIND) * w.queueCap;
	// each warp takes 32 queued pairs at a time; the sorted queues (refresh path
	// first, full path last) are taken from the back, so the long pairs start first
	const uint32_t lane = threadIdx.x & 31;
	for(;;)
	{
		uint32_t base = 0;
		if(lane == 0) base = atomicAdd(&w.workCounter[WC_NP_TAKEN + KIND], 32u);
		base = __shfl_sync(0xffffffffu, base, 0);
		if(base >= count) break;
		// lanes past the end wait at the next iteration's shuffle for the others
		if(base + lane >= count) continue;
		const uint32_t q = sorted ? count - 1u - (base + lane) : base + lane;
		const uint32_t slot = queue[q];
		const uint32_t sid = w.slotScene[slot];
		const SceneDesc sc = w.scenes[sid];
		const uint32_t key = w.pairs[slot];
		const uint32_t i = key >> 16, j = key & 0xffffu;
		// persistent mode: the pair's place in last step's (sorted) list
		uint32_t prev = NO_PREV, par = 0;
		if(sp.persistent)
		{
			par = w.sceneParity[sid];
			uint32_t lo = 0, hi = w.pairCountPrev[sid];
			const uint32_t* pk = w.pairsPrev + sc.pairStart;
			while(lo < hi)
			{
				const uint32_t mid = (lo + hi) >> 1;
				if(pk[mid] < key) lo = mid + 1;
				else hi = mid;
			}
			if(lo < w.pairCountPrev[sid] && pk[lo] == key) prev = lo;
			w.prevSlot[slot] = prev;
		}
		int ta, tb;
		float ga[4], gb[4];
		Tr pa, pb;
		pairShape(w, sc, i, ta, ga, pa);
		pairShape(w, sc, j, tb, gb, pb);
		const bool swap = ta > tb;
		np::Buffer buf;
		np::Manifold m;
		constexpr bool CACHED = (TA == 1 && (TB == 2 || TB == 3)) || (TA == 2 && TB == 3) || (TA == 3 && TB == 3);
		if(CACHED && sp.persistent && prev != NO_PREV) np::loadManifold(w.manifolds[par][sc.pairStart + prev], m);
		if(swap) generateKind<TA, TB>(gb, ga, pb, pa, sp, m, buf);
		else generateKind<TA, TB>(ga, gb, pa, pb, sp, m, buf);
		if(sp.persistent)
		{
			if(CACHED) np::storeManifold(m, w.manifolds[par ^ 1u][slot]);
			w.frictionState[par ^ 1u][slot].count = 0;   // the row preparation writes a constraint's patches
		}
		float4* o = w.contacts + size_t(slot) * 8;
		for(int c = 0; c < buf.count; c++)
		{
			V3 nn = buf.c[c].n;
			if(swap) nn = neg(nn);
			o[2 * c] = make_float4(nn.x, nn.y, nn.z, buf.c[c].sep);
			o[2 * c + 1] = make_float4(buf.c[c].p.x, buf.c[c].p.y, buf.c[c].p.z, 0.0f);
		}
		w.contactCount[slot] = uint32_t(buf.count);
	}
}

// Shared-memory workspace of the batching of one scene: batching state per
// solver body and constraint (on chip when the scene fits CAPB bodies and CAPC
// constraints) and the partition offsets.  Warp groups use SOLVE_SMEM_*,
// block groups (large scenes) BIG_SOLVE_*.
constexpr uint32_t SOLVE_SMEM_BODIES = 544;
constexpr uint32_t SOLVE_SMEM_CONSTRAINTS = 1024;
constexpr uint32_t BIG_SOLVE_BODIES = 4160;
constexpr uint32_t BIG_SOLVE_CONSTRAINTS = 8192;
template <uint32_t CAPB, uint32_t CAPC>
struct SolveSmemT
{
	uint32_t progress[CAPB];        // partition bits of the current round
	uint32_t maxNormal[CAPB];       // 1 + last dynamic partition of the body
	uint32_t maxStatic[CAPB];       // static constraints of the body
	uint32_t staticProgress[CAPB];
	uint32_t perPart[MAX_PARTITIONS];            // constraints per partition, then end offsets
	uint32_t keys[CAPC];                         // pair key of each constraint, in constraint order
	uint16_t tags[CAPC];                         // (round << 8) | partition; 0x8000 | rank for static constraints
	uint32_t bucket[MAX_PARTITIONS * 4];         // (partition, placement round) counts, then offsets
	uint32_t scan[32];
	uint32_t red, bc;
};
using SolveSmem = SolveSmemT<SOLVE_SMEM_BODIES, SOLVE_SMEM_CONSTRAINTS>;
using SolveSmemBig = SolveSmemT<BIG_SOLVE_BODIES, BIG_SOLVE_CONSTRAINTS>;

// Maximum of v over the group (slot: shared scratch word).
template <uint32_t G>
__device__ __forceinline__ uint32_t groupMax(uint32_t v, uint32_t* slot)
{
	for(int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
	if constexpr(G == 1) return v;
	else
	{
		if(threadIdx.x == 0) *slot = 0;
		__syncthreads();
		if((threadIdx.x & 31) == 0) atomicMax(slot, v);
		__syncthreads();
		const uint32_t r = *slot;
		__syncthreads();
		return r;
	}
}

// PxBatchConstraintsTGS partition rule for one scene (the rule is sequential
// in constraint order; batching.h cites the reference): one lane walks the
// constraints, the group does the parallel bookkeeping.  Fills ordered[] (pair
// indices in solve order) and the partition end offsets in perPart; returns
// the partition count (all lanes), 0 on overflow.
template <uint32_t G, uint32_t CAPB, uint32_t CAPC>
__device__ uint32_t sceneBatch(const WorldDev& w, const SceneDesc& sc, uint32_t nc, SolveSmemT<CAPB, CAPC>& sm)
{
	constexpr uint32_t NT = Grp<G>::NT;
	const uint32_t tid = Grp<G>::tid(), lane = threadIdx.x & 31;
	const uint32_t n = sc.nbBodies;
	const bool onChip = n + sc.nbStatics <= CAPB;
	uint32_t* progress = onChip ? sm.progress : w.progress + sc.solverStart;
	uint32_t* maxNormal = onChip ? sm.maxNormal : w.maxNormal + sc.solverStart;
	uint32_t* maxStatic = onChip ? sm.maxStatic : w.maxStatic + sc.solverStart;
	uint32_t* staticProgress = onChip ? sm.staticProgress : w.staticProgress + sc.solverStart;
	uint32_t* perPart = sm.perPart;
	const uint32_t* cons = w.consList + sc.pairStart;
	uint32_t* ordered = w.ordered + sc.pairStart;
	// the walk below is sequential: its operands sit in shared memory when they fit
	const bool consOnChip = nc <= CAPC;
	for(uint32_t b = tid; b < n; b += NT) { progress[b] = 0; maxNormal[b] = 0; maxStatic[b] = 0; staticProgress[b] = 0; }
	for(uint32_t p = tid; p < MAX_PARTITIONS; p += NT) perPart[p] = 0;
	if(consOnChip)
		for(uint32_t c = tid; c < nc; c += NT) { sm.keys[c] = w.pairs[sc.pairStart + cons[c]]; sm.tags[c] = 0; }
	else
		for(uint32_t c = tid; c < nc; c += NT) w.tag[sc.pairStart + c] = 0;
	Grp<G>::sync();
	auto keyOf = [&](uint32_t c) { return consOnChip ? sm.keys[c] : w.pairs[sc.pairStart + cons[c]]; };
	auto getTag = [&](uint32_t c) { return consOnChip ? uint32_t(sm.tags[c]) : w.tag[sc.pairStart + c]; };
	auto setTag = [&](uint32_t c, uint32_t t) { if(consOnChip) sm.tags[c] = uint16_t(t); else w.tag[sc.pairStart + c] = t; };
	// pass 1: dynamic-dynamic constraints take the lowest free partition bit;
	// constraints that find none retry in the next round of 32 partitions
	uint32_t nbPart = 0, maxRound = 0, fail = 0;
	if(tid == 0)
	{
		for(uint32_t round = 0;; round++)
		{
			if(round) for(uint32_t b = 0; b < n; b++) progress[b] = 0;
			bool deferred = false;
			for(uint32_t c = 0; c < nc; c++)
			{
				const uint32_t key = keyOf(c);
				const uint32_t a = key >> 16, b = key & 0xffffu;
				if(a < n && b < n)
				{
					if((getTag(c) >> 8) != round) continue;
					const uint32_t mask = ~progress[a] & ~progress[b];
					if(!mask) { setTag(c, (round + 1) << 8); deferred = true; continue; }
					const uint32_t part = __ffs(mask) - 1;
					progress[a] |= 1u << part;
					progress[b] |= 1u << part;
					const uint32_t gp = round * 32 + part;
					if(gp >= MAX_PARTITIONS) { fail = 1; break; }
					setTag(c, (round << 8) | gp);
					perPart[gp]++;
					maxNormal[a] = max(maxNormal[a], gp + 1);
					maxNormal[b] = max(maxNormal[b], gp + 1);
					nbPart = max(nbPart, gp + 1);
					maxRound = max(maxRound, round);
				}
				else if(round == 0)
				{
					// static constraint: tagged with its rank among the body's static constraints
					const uint32_t d = a < n ? a : b;
					setTag(c, 0x8000u | min(maxStatic[d], 0x7fffu));
					maxStatic[d]++;
				}
			}
			if(fail || !deferred) break;
		}
	}
	Grp<G>::sync();
	fail = Grp<G>::bcast(fail, &sm.bc);
	if(fail) return 0;
	nbPart = Grp<G>::bcast(nbPart, &sm.bc);
	maxRound = Grp<G>::bcast(maxRound, &sm.bc);
	// statics of a body follow its last dynamic partition, one per partition
	uint32_t need = nbPart;
	for(uint32_t b = tid; b < n; b += NT)
	{
		const uint32_t mn = maxNormal[b], ms = maxStatic[b];
		need = max(need, mn + ms);
		if(mn + ms <= MAX_PARTITIONS)
			for(uint32_t k = 0; k < ms; k++) atomicAdd(&perPart[mn + k], 1u);
	}
	need = groupMax<G>(need, &sm.red);
	if(need > MAX_PARTITIONS) return 0;
	nbPart = need;
	Grp<G>::sync();
	groupExclusiveScan<G>(perPart, nbPart, sm.scan);
	// pass 2: a static constraint goes to partition maxNormal[body] + its rank
	// among the body's static constraints; within a partition the reference
	// places round-0 and static constraints in input order, then each later
	// round's constraints in input order.  That is a stable counting sort by
	// (partition, placement round): counts by the group, placement by one warp.
	uint32_t* bucket = sm.bucket;
	const uint32_t nbBuckets = nbPart * 4;
	for(uint32_t i = tid; i < nbBuckets; i += NT) bucket[i] = 0;
	Grp<G>::sync();
	auto bucketOf = [&](uint32_t c) -> uint32_t {
		const uint32_t t = getTag(c);
		if(t & 0x8000u)
		{
			const uint32_t key = keyOf(c);
			const uint32_t a = key >> 16, b = key & 0xffffu;
			return (maxNormal[a < n ? a : b] + (t & 0x7fffu)) * 4;
		}
		return (t & 0xffu) * 4 + (t >> 8);
	};
	for(uint32_t c = tid; c < nc; c += NT) atomicAdd(&bucket[bucketOf(c)], 1u);
	Grp<G>::sync();
	groupExclusiveScan<G>(bucket, nbBuckets, sm.scan);
	if(Grp<G>::warp() == 0)
	for(uint32_t base = 0; base < nc; base += 32)
	{
		const uint32_t c = base + lane;
		const bool valid = c < nc;
		const uint32_t b = valid ? bucketOf(c) : 0xffffffffu;
		const uint32_t peers = __match_any_sync(0xffffffffu, b);
		const uint32_t start = valid ? bucket[b] : 0;
		__syncwarp();
		if(valid)
		{
			ordered[start + __popc(peers & laneMaskLt())] = cons[c];
			if(lane == uint32_t(__ffs(peers) - 1)) bucket[b] = start + __popc(peers);
		}
		__syncwarp();
	}
	Grp<G>::sync();
	// partition end offsets
	uint32_t endv[MAX_PARTITIONS / 32];
	for(uint32_t p = tid, k = 0; p < nbPart; p += NT, k++) endv[k] = p + 1 < nbPart ? perPart[p + 1] : nc;
	Grp<G>::sync();
	for(uint32_t p = tid, k = 0; p < nbPart; p += NT, k++) perPart[p] = endv[k];
	Grp<G>::sync();
	return nbPart;
}

// Solver bodies, constraint list and batching of one scene; queues the
// scene's constraints for row preparation.
template <uint32_t G, uint32_t CAPB, uint32_t CAPC>
__device__ __forceinline__ void sceneBatchStage(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp, SolveSmemT<CAPB, CAPC>& sm)
{
	constexpr uint32_t NT = Grp<G>::NT;
	const uint32_t tid = Grp<G>::tid(), lane = threadIdx.x & 31;
	const uint32_t n = sc.nbBodies, nTot = n + sc.nbStatics;
	tgs::BodyVel* vel = w.vel + sc.solverStart;
	tgs::BodyTx* tx = w.tx + sc.solverStart;
	tgs::BodyData* data = w.data + sc.solverStart;
	Tr* pose = w.pose + sc.solverStart;
	const V3 g = v3(sp.gx, sp.gy, sp.gz);
	// 1. solver bodies (PxConstructSolverBodiesTGS / PxConstructStaticSolverBodyTGS)
	for(uint32_t i = tid; i < nTot; i += NT)
	{
		if(i < n)
		{
			Tr p;
			tgs::constructDynamicBody(w.bodies[sc.bodyStart + i], g, sp.dt, vel[i], tx[i], data[i], p);
			pose[i] = p;
		}
		else
		{
			const Tr p = loadStaticPose(w.staticPose + 7 * size_t(sc.staticStart + (i - n)));
			tgs::constructStaticBody(p, vel[i], tx[i], data[i]);
			pose[i] = p;
		}
	}
	// 2. constraints = pairs with contacts, in pair order
	const uint32_t count = w.pairCount[sid];
	uint32_t nc = 0;
	if(Grp<G>::warp() == 0)   // in pair order: one warp
		for(uint32_t base = 0; base < count; base += 32)
		{
			const uint32_t k = base + lane;
			const bool has = k < count && w.contactCount[sc.pairStart + k] > 0;
			const uint32_t bal = __ballot_sync(0xffffffffu, has);
			if(has) w.consList[sc.pairStart + nc + __popc(bal & laneMaskLt())] = k;
			nc += __popc(bal);
		}
	Grp<G>::sync();
	nc = Grp<G>::bcast(nc, &sm.bc);
	// 3. batching
	const uint32_t nbPart = sceneBatch<G>(w, sc, nc, sm);
	for(uint32_t p = tid; p < nbPart; p += NT) w.partEnds[size_t(sid) * MAX_PARTITIONS + p] = sm.perPart[p];
	if(tid == 0)
	{
		w.nbConstraints[sid] = nc;
		w.nbPartitions[sid] = nbPart;
		if(!nbPart && nc) atomicOr(&w.status[sid], ST_PARTITION_OVERFLOW);
		if(sp.solveVariant == RESIDENT_VARIANT)
		{
			// the row preparation files scenes with constraints once their last row is built
			w.sceneAcc[sid] = 0;
			if(!nbPart) residentAppend(w, sid, residentLevel(residentBytes(0, nTot, 0), sp.resBytes));
		}
	}
	if(!nbPart) return;   // nothing to solve, or overflow: the scene is left unchanged
	uint32_t qbase = 0;
	if(tid == 0) qbase = atomicAdd(&w.workCounter[3], nc);
	qbase = Grp<G>::bcast(qbase, &sm.bc);
	// PxBatchConstraintsTGS's headers are runs of up to 4 consecutive constraints
	// of one partition (createHeaders, NpImmediateMode.cpp:159; every partition
	// here is non-empty, so each one is below its maxPartition); full runs of 4
	// take the 4-wide block path (<= 16 contacts, under its 64-contact limit).
	// Bit 31 of the queue entry marks those constraints.
	for(uint32_t r = tid; r < nc; r += NT)
	{
		uint32_t lo = 0, hi = nbPart - 1;   // first partition whose end is above r
		while(lo < hi)
		{
			const uint32_t mid = (lo + hi) >> 1;
			if(sm.perPart[mid] > r) hi = mid;
			else lo = mid + 1;
		}
		const uint32_t start = lo ? sm.perPart[lo - 1] : 0u, size = sm.perPart[lo] - start;
		const bool block = (r - start) < (size & ~3u);
		w.prepQueue[qbase + r] = (sc.pairStart + r) | (block ? 0x80000000u : 0u);
		// class: the path, the contact count and last step's friction patches, so that
		// a warp of the preparation runs one code path
		const uint32_t k = w.ordered[sc.pairStart + r];
		const uint32_t cnt = w.contactCount[sc.pairStart + k];
		uint32_t prevPatches = 0;
		if(sp.persistent)
		{
			const uint32_t prev = w.prevSlot[sc.pairStart + k];
			if(prev != NO_PREV) prevPatches = w.frictionState[w.sceneParity[sid]][sc.pairStart + prev].count;
		}
		const uint32_t cls = (block ? 16u : 0u) | (((cnt - 1u) & 3u) << 2) | (prevPatches < 3u ? prevPatches : 3u);
		w.prepClass[qbase + r] = uint8_t(cls);
		const uint32_t peers = __match_any_sync(__activemask(), cls);
		if((threadIdx.x & 31) == uint32_t(__ffs(peers) - 1)) atomicAdd(&w.workCounter[WC_PREP_CLASS + cls], uint32_t(__popc(peers)));
	}
}

// The preparation queue grouped by class (a stable order is not needed: every
// constraint's rows go to its own slot).
__global__ void __launch_bounds__(128) prepOrderKernel(WorldDev w, StepParams sp)
{
	__shared__ uint32_t first[PREP_CLASSES];
	if(threadIdx.x < 32)
	{
		const uint32_t c = w.workCounter[WC_PREP_CLASS + threadIdx.x];
		uint32_t incl = c;
		for(int d = 1; d < 32; d <<= 1)
		{
			const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
			if(threadIdx.x >= uint32_t(d)) incl += t;
		}
		first[threadIdx.x] = incl - c;
	}
	__syncthreads();
	const uint32_t count = w.workCounter[WC_PREP];
	const uint32_t lane = threadIdx.x & 31;
	for(uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x)
	{
		const uint32_t q = base + threadIdx.x;
		const bool valid = q < count;
		const uint32_t cls = valid ? uint32_t(w.prepClass[q]) : 0xffu;
		const uint32_t peers = __match_any_sync(0xffffffffu, cls);
		const uint32_t leader = __ffs(peers) - 1;
		uint32_t b = 0;
		if(valid && lane == leader) b = atomicAdd(&w.workCounter[WC_PREP_PLACED + cls], uint32_t(__popc(peers)));
		b = __shfl_sync(0xffffffffu, b, leader);
		if(valid) w.prepQueueSorted[first[cls] + b + __popc(peers & laneMaskLt())] = w.prepQueue[q];
	}
}

// Contact rows of one constraint (PxCreateContactConstraintsTGS for one
// descriptor): slot = scene pair start + position in solve order.
__device__ __forceinline__ uint32_t prepSlot(const WorldDev& w, uint32_t entry, const StepParams& sp)
{
	const uint32_t slot = entry & 0x7fffffffu;
	const bool block = (entry >> 31) != 0;
	const SceneDesc sc = w.scenes[w.slotScene[slot]];
	const uint32_t n = sc.nbBodies;
	tgs::BodyVel* vel = w.vel + sc.solverStart;
	tgs::BodyTx* tx = w.tx + sc.solverStart;
	tgs::BodyData* data = w.data + sc.solverStart;
	Tr* pose = w.pose + sc.solverStart;
	const tgs::PrepParams pp = prepParams(sp);
	const uint32_t k = w.ordered[slot];
	const uint32_t key = w.pairs[sc.pairStart + k];
	const uint32_t a = key >> 16, b = key & 0xffffu;
	const float fa = w.friction[sc.bodyStart + a];
	const float fb = b < n ? w.friction[sc.bodyStart + b] : sp.staticFriction;
	const float mu = (fa + fb) * 0.5f;
	tgs::Contact cs[tgs::MAX_CONTACTS];
	const uint32_t cnt = w.contactCount[sc.pairStart + k];
	const float4* src = w.contacts + size_t(sc.pairStart + k) * 8;
	for(uint32_t c = 0; c < cnt; c++)
	{
		const float4 nn = src[2 * c], pp4 = src[2 * c + 1];
		cs[c].n = v3(nn.x, nn.y, nn.z);
		cs[c].sep = nn.w;
		cs[c].p = v3(pp4.x, pp4.y, pp4.z);
		cs[c].staticFriction = mu;
		cs[c].dynamicFriction = mu;
		cs[c].restitution = 0.0f;
	}
	tgs::ConstraintRecord& rec = w.recs[slot];
	const tgs::FrictionState* prevFriction = nullptr;
	tgs::FrictionState* written = nullptr;
	if(sp.persistent)
	{
		const uint32_t par = w.sceneParity[w.slotScene[slot]];
		const uint32_t prev = w.prevSlot[sc.pairStart + k];
		if(prev != NO_PREV) prevFriction = w.frictionState[par] + sc.pairStart + prev;
		written = w.frictionState[par ^ 1u] + sc.pairStart + k;
	}
	if(block)
		tgs::prepConstraintBlock(cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, b < n, b == 0,
		                         rec, prevFriction, written);
	else
		tgs::prepConstraint(cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, rec, prevFriction,
		                    written);
	const uint32_t chunks = (rec.bytes() + 15) / 16;
	w.recChunks[slot] = uint8_t(chunks);
	return chunks;
}

// Counts a prepared constraint towards its scene; the scene's last one files
// the scene for the resident solve at the level its footprint fits.
__device__ __forceinline__ void residentCount(const WorldDev& w, uint32_t slot, uint32_t chunks, const StepParams& sp)
{
	const uint32_t sid = w.slotScene[slot];
	const unsigned long long old = atomicAdd(&w.sceneAcc[sid], (1ull << 32) | chunks);
	const uint32_t nc = w.nbConstraints[sid];
	if(uint32_t(old >> 32) + 1u == nc)
	{
		const SceneDesc sc = w.scenes[sid];
		const uint32_t nTot = sc.nbBodies + sc.nbStatics;
		uint32_t level = residentLevel(residentBytes(nc, nTot, uint32_t(old) + chunks), sp.resBytes);
		// streamed rows: a scene filed above level resStream goes one level deeper
		// (groups of two warps at least), so more scenes are in flight per SM
		if(level < sp.resStream && level + 2 < RES_LEVELS && residentStreamBytes(nc, nTot) <= (sp.resBytes >> (level + 1))) level++;
		residentAppend(w, sid, level);
	}
}

// Velocities of one scene's solver bodies during the iterations: linear and
// (momentum-space) angular velocity, the values every constraint solve
// reads and writes.  Scenes that fit the workspace keep them in shared
// memory; larger scenes use the BodyVel records in HBM.
struct SharedVel
{
	V3* l;
	V3* a;
	__device__ __forceinline__ V3 lin(uint32_t i) const { return l[i]; }
	__device__ __forceinline__ V3 ang(uint32_t i) const { return a[i]; }
	__device__ __forceinline__ void set(uint32_t i, V3 lv, V3 av) const { l[i] = lv; a[i] = av; }
};
struct GlobalVel
{
	tgs::BodyVel* v;
	__device__ __forceinline__ V3 lin(uint32_t i) const { return v[i].lin; }
	__device__ __forceinline__ V3 ang(uint32_t i) const { return v[i].ang; }
	__device__ __forceinline__ void set(uint32_t i, V3 l, V3 a) const { v[i].lin = l; v[i].ang = a; }
};

// Position iterations (each followed by integration), velocity iterations,
// PxIntegrateSolverBodiesTGS and write-back of one scene.
// In warp groups each lane stages the packed rows of the constraint it solves
// in shared memory with asynchronous 16-byte copies (one memory round trip per
// constraint instead of one per row), solves from there and writes the updated
// impulses back; rows larger than the staging slot, and the rows of block
// groups (large scenes), are used in place.
constexpr uint32_t RECBUF_CHUNKS = 32;   // 512 bytes per lane
template <uint32_t CAPB, uint32_t CAPC, uint32_t RB>
struct __align__(16) IterSmemT
{
	float4 recBuf[RB ? 32 : 1][RB + 1];   // RB 16-byte chunks per lane, padded: lanes' slots start in different banks
	V3 lin[CAPB], ang[CAPB];
	uint32_t ends[MAX_PARTITIONS];
	uint8_t chunks[CAPC];
	uint32_t bc;
};
// Warp-per-scene solve variants: staging slot (chunks of 16 bytes per lane) and
// whether the body velocities sit in shared memory (CAPB = SOLVE_SMEM_BODIES) or
// stay in HBM/L1 (CAPB = 1).  Smaller workspaces leave room for more warps per SM.
template <uint32_t CAPB, uint32_t RB>
using IterSmemW = IterSmemT<CAPB, SOLVE_SMEM_CONSTRAINTS, RB>;
using IterSmemBig = IterSmemT<BIG_SOLVE_BODIES, BIG_SOLVE_CONSTRAINTS, 0>;
// variants: (velocities on chip, 0 / 256 / 512 B staging), (velocities in HBM, 0 / 256 / 512 B), then 400 B
// staging with velocities on chip / in HBM (the largest slot that leaves room for 8 warps per SM with
// the velocities on chip; one-patch four-point rows are 392 B)
constexpr uint32_t SOLVE_VARIANTS = 8;
static_assert(RESIDENT_VARIANT == SOLVE_VARIANTS, "the resident solve follows the staging variants");
constexpr uint32_t MID_CHUNKS = 25;

template <uint32_t G, uint32_t CAPB, uint32_t CAPC, uint32_t RB, typename Vel>
__device__ __forceinline__ void sceneIterate(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp,
                                             IterSmemT<CAPB, CAPC, RB>& sm, uint32_t nbPart, const Vel& V)
{
	constexpr uint32_t NT = Grp<G>::NT;
	const uint32_t tid = Grp<G>::tid();
	const uint32_t n = sc.nbBodies, nTot = n + sc.nbStatics;
	const uint32_t* ends = sm.ends;
	tgs::BodyVel* vel = w.vel + sc.solverStart;
	tgs::BodyTx* tx = w.tx + sc.solverStart;
	Tr* pose = w.pose + sc.solverStart;
	const uint32_t nc = nbPart ? ends[nbPart - 1] : 0;
	const bool chunksOnChip = RB > 0 && nc <= CAPC;
	if(chunksOnChip)
		for(uint32_t r = tid; r < nc; r += NT) sm.chunks[r] = w.recChunks[sc.pairStart + r];
	for(uint32_t i = tid; i < nTot; i += NT) V.set(i, vel[i].lin, vel[i].ang);
	Grp<G>::sync();
	const float stepDt = sp.dt / float(sp.nbPos);
	float elapsed = 0.0f;
	for(uint32_t it = 0; it < sp.nbPos + sp.nbVel; it++)
	{
		const bool posIter = it < sp.nbPos;
		const float minPen = posIter ? -FLT_MAX : 0.0f;
		uint32_t begin = 0;
		for(uint32_t p = 0; p < nbPart; p++)
		{
			const uint32_t end = ends[p];
			for(uint32_t r = begin + tid; r < end; r += NT)
			{
				tgs::ConstraintRecord* src = w.recs + sc.pairStart + r;
				tgs::ConstraintRecord* rec = src;
				if constexpr(RB > 0)
				{
					const uint32_t chunks = chunksOnChip ? sm.chunks[r] : w.recChunks[sc.pairStart + r];
					if(chunks <= RB)
					{
						float4* dst = sm.recBuf[threadIdx.x & 31];
						const float4* g = reinterpret_cast<const float4*>(src);
						for(uint32_t k = 0; k < chunks; k++) cpAsync16(dst + k, g + k);
						cpAsyncWaitAll();
						rec = reinterpret_cast<tgs::ConstraintRecord*>(dst);
					}
				}
				if(rec->nbPatches == 0) continue;
				const uint32_t a = uint32_t(rec->bodyA), b = uint32_t(rec->bodyB);
				tgs::BodyVel b0, b1;
				b0.lin = V.lin(a); b0.ang = V.ang(a); b0.dLin = vel[a].dLin; b0.dAng = vel[a].dAng;
				b1.lin = V.lin(b); b1.ang = V.ang(b); b1.dLin = vel[b].dLin; b1.dAng = vel[b].dAng;
				const bool dynB = b < n;
				const bool lastIter = it + 1 == sp.nbPos + sp.nbVel;
				uint32_t broken = 0;
				tgs::solveRecord(*rec, b0, b1, dynB, minPen, elapsed, sp.persistent && lastIter ? &broken : nullptr);
				if(broken)
				{
					// write-back of the last iteration: a patch whose friction was
					// clamped marks the friction patch it wrote broken
					tgs::FrictionState& fs = w.frictionState[w.sceneParity[sid] ^ 1u][sc.pairStart + w.ordered[sc.pairStart + r]];
					tgs::ConstraintRecord* group[4] = {nullptr, nullptr, nullptr, nullptr};
					if(rec->isBlock())
					{
						const uint32_t r0 = begin + ((r - begin) & ~3u);
						for(uint32_t l = 0; l < 4; l++) group[l] = w.recs + sc.pairStart + r0 + l;
					}
					for(int pi = 0; pi < rec->nbPatches; pi++)
						if(broken & (1u << pi))
						{
							const int slotIdx = rec->isBlock() ? tgs::blockBrokenSlot(group, pi) : pi;
							if(uint32_t(slotIdx) < fs.count) fs.patches[slotIdx].broken = 1;
						}
				}
				V.set(a, b0.lin, b0.ang);
				if(dynB) V.set(b, b1.lin, b1.ang);
				if(rec != src)
				{
					// the impulses are the only rows the solve updates
					const float* f = rec->force();
					float* gf = src->force();
					const int nf = rec->nbPoints() + rec->nbFriction();
					for(int k = 0; k < nf; k++) gf[k] = f[k];
				}
			}
			begin = end;
			Grp<G>::sync();
		}
		if(posIter)
		{
			for(uint32_t i = tid; i < n; i += NT)
			{
				tgs::BodyVel v = vel[i];
				v.lin = V.lin(i);
				v.ang = V.ang(i);
				tgs::integrateStep(v, tx[i], stepDt);
				vel[i].dLin = v.dLin;
				vel[i].dAng = v.dAng;
			}
			elapsed += stepDt;
			Grp<G>::sync();
		}
	}
	for(uint32_t i = tid; i < n; i += NT)
	{
		tgs::BodyVel v = vel[i];
		v.lin = V.lin(i);
		v.ang = V.ang(i);
		Tr p = pose[i];
		V3 wv;
		tgs::finalizeBody(v, tx[i], p, wv);
		tgs::RigidBody& rb = w.bodies[sc.bodyStart + i];
		rb.linVel[0] = v.lin.x; rb.linVel[1] = v.lin.y; rb.linVel[2] = v.lin.z;
		rb.angVel[0] = wv.x; rb.angVel[1] = wv.y; rb.angVel[2] = wv.z;
		rb.q[0] = p.q.x; rb.q[1] = p.q.y; rb.q[2] = p.q.z; rb.q[3] = p.q.w;
		rb.p[0] = p.p.x; rb.p[1] = p.p.y; rb.p[2] = p.p.z;
	}
	Grp<G>::sync();
}

// Stage kernels of one step.  The scene stages (broadphase, batching, solve)
// run persistent grids that pull scenes from the size-sorted work table
// (largest first): warp-per-scene kernels take the scenes of up to
// sp.largeBodies solver bodies, block-per-scene kernels (BIG_WARPS warps, the
// workspace for up to 4096 bodies on chip) the larger ones.  The narrowphase
// runs one kernel per pair kind over all scenes' pairs.
__device__ __forceinline__ bool largeScene(const SceneDesc& sc, const StepParams& sp) { return sc.nbBodies + sc.nbStatics > sp.largeBodies; }

// Next scene of the wanted size class from work counter `counter` (all threads of
// the group get it); false when the table is exhausted.
template <uint32_t G>
__device__ __forceinline__ bool nextScene(const WorldDev& w, uint32_t counter, bool wantLarge, const StepParams& sp, uint32_t& sid,
                                          SceneDesc& sc, volatile uint32_t* slot)
{
	for(;;)
	{
		uint32_t item = 0;
		if(Grp<G>::tid() == 0) item = atomicAdd(&w.workCounter[counter], 1u);
		item = Grp<G>::bcast(item, slot);
		if(item >= *w.nbActive) return false;
		sid = w.workOrder[item];
		sc = w.scenes[sid];
		if(largeScene(sc, sp) == wantLarge) return true;
	}
}


__global__ void __launch_bounds__(128) broadphaseKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	BpSmem& sm = reinterpret_cast<BpSmem*>(stageSmem)[threadIdx.x >> 5];
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<1>(w, WC_BP, false, sp, sid, sc, nullptr)) sceneBroadphase<1>(w, sc, sid, sp, sm);
}

__global__ void __launch_bounds__(BIG_WARPS * 32) broadphaseBigKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	BpSmemBig& sm = *reinterpret_cast<BpSmemBig*>(stageSmem);
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<BIG_WARPS>(w, WC_BP_BIG, true, sp, sid, sc, &sm.bc)) sceneBroadphase<BIG_WARPS>(w, sc, sid, sp, sm);
}

__global__ void __launch_bounds__(128) batchKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	SolveSmem& sm = reinterpret_cast<SolveSmem*>(stageSmem)[threadIdx.x >> 5];
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<1>(w, WC_BATCH, false, sp, sid, sc, nullptr)) sceneBatchStage<1>(w, sc, sid, sp, sm);
}

__global__ void __launch_bounds__(BIG_WARPS * 32) batchBigKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	SolveSmemBig& sm = *reinterpret_cast<SolveSmemBig*>(stageSmem);
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<BIG_WARPS>(w, WC_BATCH_BIG, true, sp, sid, sc, &sm.bc)) sceneBatchStage<BIG_WARPS>(w, sc, sid, sp, sm);
}

// Row preparation of every scene's constraints: a thread per constraint.
__global__ void __launch_bounds__(128, 5) prepKernel(WorldDev w, StepParams sp)
{
	const uint32_t count = w.workCounter[WC_PREP];
	for(uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x)
	{
		const uint32_t entry = w.prepQueueSorted[q];
		const uint32_t chunks = prepSlot(w, entry, sp);
		if(sp.solveVariant == RESIDENT_VARIANT) residentCount(w, entry & 0x7fffffffu, chunks, sp);
	}
}

// Iterations of one scene; afterwards the state this step wrote becomes the
// scene's last-step state.
template <uint32_t G, uint32_t CAPB, uint32_t CAPC, uint32_t RB>
__device__ __forceinline__ void solveScene(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp,
                                           IterSmemT<CAPB, CAPC, RB>& sm)
{
	const uint32_t tid = Grp<G>::tid();
	const uint32_t nbPart = w.nbPartitions[sid];
	if(nbPart || !w.nbConstraints[sid])   // batching overflowed: the scene is left unchanged
	{
		for(uint32_t p = tid; p < nbPart; p += Grp<G>::NT) sm.ends[p] = w.partEnds[size_t(sid) * MAX_PARTITIONS + p];
		Grp<G>::sync();
		if(sc.nbBodies + sc.nbStatics <= CAPB) sceneIterate<G>(w, sc, sid, sp, sm, nbPart, SharedVel{sm.lin, sm.ang});
		else sceneIterate<G>(w, sc, sid, sp, sm, nbPart, GlobalVel{w.vel + sc.solverStart});
	}
	Grp<G>::sync();
	if(sp.persistent && tid == 0) w.sceneParity[sid] ^= 1u;
}

constexpr uint32_t SOLVE_WARPS = 1;   // warps (scenes in flight) per block of the warp-per-scene solve kernel
template <uint32_t CAPB, uint32_t RB>
__global__ void __launch_bounds__(SOLVE_WARPS * 32) solveKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	IterSmemW<CAPB, RB>& sm = reinterpret_cast<IterSmemW<CAPB, RB>*>(stageSmem)[threadIdx.x >> 5];
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<1>(w, WC_SOLVE, false, sp, sid, sc, nullptr)) solveScene<1>(w, sc, sid, sp, sm);
}

__global__ void __launch_bounds__(BIG_WARPS * 32) solveBigKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char stageSmem[];
	IterSmemBig& sm = *reinterpret_cast<IterSmemBig*>(stageSmem);
	uint32_t sid;
	SceneDesc sc;
	while(nextScene<BIG_WARPS>(w, WC_SOLVE_BIG, true, sp, sid, sc, &sm.bc)) solveScene<BIG_WARPS>(w, sc, sid, sp, sm);
}

// ------------------------------------------------------------------ resident solve
// Shared-memory barrier (mbarrier) and bulk-copy primitives (PTX, sm_90+).
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbarInit(unsigned long long* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarArriveExpectTx(unsigned long long* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbarTryWait(unsigned long long* bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.b32 %0, 1, 0, P;\n}\n"
	             : "=r"(ok)
	             : "r"(smemAddr(bar)), "r"(parity)
	             : "memory");
	return ok != 0;
}
// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from
// this GPU's global memory into this block's shared memory, completing on `bar`.
__device__ __forceinline__ void bulkCopyToShared(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(smemAddr(dst)), "l"(src),
	             "r"(bytes), "r"(smemAddr(bar))
	             : "memory");
}
// Orders this thread's earlier shared-memory accesses before later bulk copies into them.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// Orders this thread's earlier global writes before later bulk copies that read them.
__device__ __forceinline__ void fenceProxyAsyncGlobal() { asm volatile("fence.proxy.async.global;\n" ::: "memory"); }
// try_wait rounds before a bulk copy counts as lost (each round may suspend the
// thread for a while; this is well above a second)
constexpr uint32_t STAGE_WAIT_LIMIT = 1u << 22;

// Barrier of the nt threads of a group (barId: named barrier of the group; one
// warp synchronises with __syncwarp).
__device__ __forceinline__ void groupSync(uint32_t barId, uint32_t nt)
{
	if(nt == 32) __syncwarp();
	else asm volatile("bar.sync %0, %1;\n" ::"r"(barId), "r"(nt) : "memory");
}

// Exclusive prefix of `sum` over a group's threads in thread order; `total`
// gets the group's sum.  scratch: one word per warp of the group.
__device__ __forceinline__ uint32_t groupPrefix(uint32_t sum, uint32_t* scratch, uint32_t gtid, uint32_t nt, uint32_t barId, uint32_t& total)
{
	const uint32_t lane = gtid & 31, gwarp = gtid >> 5;
	uint32_t incl = sum;
	for(int o = 1; o < 32; o <<= 1)
	{
		const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= uint32_t(o)) incl += t;
	}
	if(lane == 31) scratch[gwarp] = incl;
	groupSync(barId, nt);
	uint32_t off = 0, tot = 0;
	for(uint32_t q = 0; q < (nt >> 5); q++)
	{
		const uint32_t v = scratch[q];
		if(q < gwarp) off += v;
		tot += v;
	}
	groupSync(barId, nt);
	total = tot;
	return off + incl - sum;
}

// Velocities of the solver bodies of a scene during the resident solve: linear,
// (momentum-space) angular and the accumulated position / rotation deltas, in
// four shared-memory arrays, or in the BodyVel records in HBM for scenes whose
// bodies do not fit the slice.
struct ResVel
{
	V3 *l, *a, *dl, *da;
	__device__ __forceinline__ V3 lin(uint32_t i) const { return l[i]; }
	__device__ __forceinline__ V3 ang(uint32_t i) const { return a[i]; }
	__device__ __forceinline__ V3 dLin(uint32_t i) const { return dl[i]; }
	__device__ __forceinline__ V3 dAng(uint32_t i) const { return da[i]; }
	__device__ __forceinline__ void set(uint32_t i, V3 lv, V3 av) const { l[i] = lv; a[i] = av; }
	__device__ __forceinline__ void setDelta(uint32_t i, V3 dlv, V3 dav) const { dl[i] = dlv; da[i] = dav; }
};
struct ResHbmVel
{
	tgs::BodyVel* v;
	__device__ __forceinline__ V3 lin(uint32_t i) const { return v[i].lin; }
	__device__ __forceinline__ V3 ang(uint32_t i) const { return v[i].ang; }
	__device__ __forceinline__ V3 dLin(uint32_t i) const { return v[i].dLin; }
	__device__ __forceinline__ V3 dAng(uint32_t i) const { return v[i].dAng; }
	__device__ __forceinline__ void set(uint32_t i, V3 lv, V3 av) const { v[i].lin = lv; v[i].ang = av; }
	__device__ __forceinline__ void setDelta(uint32_t i, V3 dlv, V3 dav) const { v[i].dLin = dlv; v[i].dAng = dav; }
};

// Position iterations (each followed by integration), velocity iterations,
// PxIntegrateSolverBodiesTGS and write-back of one scene by a group of nt
// threads: the arithmetic of sceneIterate.  ROWS_ON_CHIP: the rows of
// constraint r sit at rows + 16 * off[r] in shared memory (the solve's impulses
// stay there: nothing reads them after the solve); otherwise they are used in
// place in HBM.
template <bool ROWS_ON_CHIP, typename Vel>
__device__ __forceinline__ void residentIterate(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp, const uint32_t* ends,
                                                uint32_t nbPart, const uint16_t* off, unsigned char* rows, const Vel& V, uint32_t gtid,
                                                uint32_t nt, uint32_t barId)
{
	const uint32_t n = sc.nbBodies;
	tgs::BodyTx* tx = w.tx + sc.solverStart;
	Tr* pose = w.pose + sc.solverStart;
	auto recAt = [&](uint32_t r) -> tgs::ConstraintRecord* {
		if constexpr(ROWS_ON_CHIP) return reinterpret_cast<tgs::ConstraintRecord*>(rows + 16u * off[r]);
		else return w.recs + sc.pairStart + r;
	};
	const float stepDt = sp.dt / float(sp.nbPos);
	float elapsed = 0.0f;
	for(uint32_t it = 0; it < sp.nbPos + sp.nbVel; it++)
	{
		const bool posIter = it < sp.nbPos;
		const bool lastIter = it + 1 == sp.nbPos + sp.nbVel;
		const float minPen = posIter ? -FLT_MAX : 0.0f;
		uint32_t begin = 0;
		for(uint32_t p = 0; p < nbPart; p++)
		{
			const uint32_t end = ends[p];
			for(uint32_t r = begin + gtid; r < end; r += nt)
			{
				tgs::ConstraintRecord* rec = recAt(r);
				if(rec->nbPatches == 0) continue;
				const uint32_t a = uint32_t(rec->bodyA), b = uint32_t(rec->bodyB);
				tgs::BodyVel b0, b1;
				b0.lin = V.lin(a); b0.ang = V.ang(a); b0.dLin = V.dLin(a); b0.dAng = V.dAng(a);
				b1.lin = V.lin(b); b1.ang = V.ang(b); b1.dLin = V.dLin(b); b1.dAng = V.dAng(b);
				const bool dynB = b < n;
				uint32_t broken = 0;
				tgs::solveRecord(*rec, b0, b1, dynB, minPen, elapsed, sp.persistent && lastIter ? &broken : nullptr);
				if(broken)
				{
					// a patch whose friction was clamped in the last iteration marks the
					// friction patch it wrote broken
					tgs::FrictionState& fs = w.frictionState[w.sceneParity[sid] ^ 1u][sc.pairStart + w.ordered[sc.pairStart + r]];
					tgs::ConstraintRecord* group[4] = {nullptr, nullptr, nullptr, nullptr};
					if(rec->isBlock())
					{
						const uint32_t r0 = begin + ((r - begin) & ~3u);
						for(uint32_t l = 0; l < 4; l++) group[l] = recAt(r0 + l);
					}
					for(int pi = 0; pi < rec->nbPatches; pi++)
						if(broken & (1u << pi))
						{
							const int slotIdx = rec->isBlock() ? tgs::blockBrokenSlot(group, pi) : pi;
							if(uint32_t(slotIdx) < fs.count) fs.patches[slotIdx].broken = 1;
						}
				}
				V.set(a, b0.lin, b0.ang);
				if(dynB) V.set(b, b1.lin, b1.ang);
			}
			begin = end;
			groupSync(barId, nt);
		}
		if(posIter)
		{
			for(uint32_t i = gtid; i < n; i += nt)
			{
				tgs::BodyVel v;
				v.lin = V.lin(i); v.ang = V.ang(i); v.dLin = V.dLin(i); v.dAng = V.dAng(i);
				tgs::integrateStep(v, tx[i], stepDt);
				V.setDelta(i, v.dLin, v.dAng);
			}
			elapsed += stepDt;
			groupSync(barId, nt);
		}
	}
	for(uint32_t i = gtid; i < n; i += nt)
	{
		tgs::BodyVel v;
		v.lin = V.lin(i); v.ang = V.ang(i); v.dLin = V.dLin(i); v.dAng = V.dAng(i);
		Tr p = pose[i];
		V3 wv;
		tgs::finalizeBody(v, tx[i], p, wv);
		tgs::RigidBody& rb = w.bodies[sc.bodyStart + i];
		rb.linVel[0] = v.lin.x; rb.linVel[1] = v.lin.y; rb.linVel[2] = v.lin.z;
		rb.angVel[0] = wv.x; rb.angVel[1] = wv.y; rb.angVel[2] = wv.z;
		rb.q[0] = p.q.x; rb.q[1] = p.q.y; rb.q[2] = p.q.z; rb.q[3] = p.q.w;
		rb.p[0] = p.p.x; rb.p[1] = p.p.y; rb.p[2] = p.p.z;
	}
}

// The iterations of residentIterate for a scene with streamed rows.  table:
// chunkFirst[0..nChunks] (first constraint of each chunk, then nc) followed by
// the first chunk of each partition; off: each constraint's row offset (16-byte
// units) from the scene's first row, total: all rows; slots: the two ring slots
// of slotBytes; bars / phase: the two slot barriers and the parity each waits
// for next.  Returns false when a bulk copy did not complete within the wait
// limit (after a bounded wait for the copies in flight).
template <typename Vel>
__device__ __forceinline__ bool residentIterateStreamed(const WorldDev& w, const SceneDesc& sc, uint32_t sid, const StepParams& sp,
                                                        const uint32_t* ends, uint32_t nbPart, const uint16_t* off, uint32_t total,
                                                        const uint32_t* chunkFirst, uint32_t nChunks, unsigned char* slot0, uint32_t slotBytes,
                                                        const Vel& V, uint32_t gtid, uint32_t nt, uint32_t barId, unsigned long long* bars,
                                                        uint32_t* phase, uint32_t* word)
{
	const uint32_t n = sc.nbBodies, nc = ends[nbPart - 1];
	tgs::BodyTx* tx = w.tx + sc.solverStart;
	Tr* pose = w.pose + sc.solverStart;
	tgs::ConstraintRecord* recs = w.recs + sc.pairStart;
	const uint32_t nIter = sp.nbPos + sp.nbVel, nSeq = nIter * nChunks;
	const uint32_t ph0 = phase[0], ph1 = phase[1];
	auto unitEnd = [&](uint32_t r) -> uint32_t { return r < nc ? uint32_t(off[r]) : total; };
	// bulk copies of chunk g of the sequence (iteration g / nChunks) into slot g & 1
	auto issue = [&](uint32_t g) {
		const uint32_t j = g % nChunks, sl = g & 1u;
		const uint32_t c0 = chunkFirst[j], c1 = chunkFirst[j + 1];
		const uint32_t u0 = off[c0];
		unsigned char* dst = slot0 + size_t(sl) * slotBytes;
		if(gtid == 0) mbarArriveExpectTx(&bars[sl], 16u * (unitEnd(c1) - u0));
		for(uint32_t r = c0 + gtid; r < c1; r += nt)
			bulkCopyToShared(dst + 16u * (off[r] - u0), recs + r, 16u * (unitEnd(r + 1) - off[r]), &bars[sl]);
	};
	// bounded wait for chunk g, voted over the group
	auto ready = [&](uint32_t g) -> bool {
		const uint32_t sl = g & 1u, parity = (sl ? ph1 : ph0) ^ ((g >> 1) & 1u);
		bool done = false;
		for(uint32_t k = 0; k < STAGE_WAIT_LIMIT && !done; k++) done = mbarTryWait(&bars[sl], parity);
		if(!__all_sync(0xffffffffu, done) && (gtid & 31) == 0) atomicOr(word, 1u);
		groupSync(barId, nt);
		return *word == 0;
	};
	auto fail = [&](uint32_t g) {
		// a copy is lost: flag the scene and give the copies in flight a last bounded wait
		if(gtid == 0) atomicOr(&w.status[sid], ST_STAGE_TIMEOUT);
		for(uint32_t h = g; h < g + 2 && h < nSeq; h++)
		{
			const uint32_t sl = h & 1u, parity = (sl ? ph1 : ph0) ^ ((h >> 1) & 1u);
			bool done = false;
			for(uint32_t k = 0; k < STAGE_WAIT_LIMIT && !done; k++) done = mbarTryWait(&bars[sl], parity);
		}
	};
	const float stepDt = sp.dt / float(sp.nbPos);
	float elapsed = 0.0f;
	uint32_t g = 0;
	issue(0);
	for(uint32_t it = 0; it < nIter; it++)
	{
		const bool posIter = it < sp.nbPos;
		const bool lastIter = it + 1 == nIter;
		const float minPen = posIter ? -FLT_MAX : 0.0f;
		for(uint32_t j = 0; j < nChunks; j++, g++)
		{
			if(!ready(g)) { fail(g); return false; }
			// slot (g + 1) & 1 held chunk g - 1, solved before the last barrier
			if(g + 1 < nSeq) issue(g + 1);
			unsigned char* base = slot0 + size_t(g & 1u) * slotBytes;
			const uint32_t c0 = chunkFirst[j], c1 = chunkFirst[j + 1], u0 = off[c0];
			for(uint32_t r = c0 + gtid; r < c1; r += nt)
			{
				tgs::ConstraintRecord* rec = reinterpret_cast<tgs::ConstraintRecord*>(base + 16u * (off[r] - u0));
				if(rec->nbPatches == 0) continue;
				const uint32_t a = uint32_t(rec->bodyA), b = uint32_t(rec->bodyB);
				tgs::BodyVel b0, b1;
				b0.lin = V.lin(a); b0.ang = V.ang(a); b0.dLin = V.dLin(a); b0.dAng = V.dAng(a);
				b1.lin = V.lin(b); b1.ang = V.ang(b); b1.dLin = V.dLin(b); b1.dAng = V.dAng(b);
				const bool dynB = b < n;
				uint32_t broken = 0;
				tgs::solveRecord(*rec, b0, b1, dynB, minPen, elapsed, sp.persistent && lastIter ? &broken : nullptr);
				// the impulses go back to the record in HBM for the next iteration's copy
				const float* src = rec->force();
				float* dst = reinterpret_cast<float*>(reinterpret_cast<char*>(recs + r) + (reinterpret_cast<const char*>(src) - reinterpret_cast<const char*>(rec)));
				const int nImp = rec->nbPoints() + rec->nbFriction();
				for(int i = 0; i < nImp; i++) dst[i] = src[i];
				if(broken)
				{
					tgs::FrictionState& fs = w.frictionState[w.sceneParity[sid] ^ 1u][sc.pairStart + w.ordered[sc.pairStart + r]];
					tgs::ConstraintRecord* group[4] = {nullptr, nullptr, nullptr, nullptr};
					if(rec->isBlock())
					{
						// the header's lanes (consecutive constraints of the partition) read in HBM:
						// only their patch and friction counts are used
						uint32_t pb = 0;
						while(ends[pb] <= r) pb++;
						const uint32_t begin = pb ? ends[pb - 1] : 0u;
						const uint32_t r0 = begin + ((r - begin) & ~3u);
						for(uint32_t l = 0; l < 4; l++) group[l] = recs + r0 + l;
					}
					for(int pi = 0; pi < rec->nbPatches; pi++)
						if(broken & (1u << pi))
						{
							const int slotIdx = rec->isBlock() ? tgs::blockBrokenSlot(group, pi) : pi;
							if(uint32_t(slotIdx) < fs.count) fs.patches[slotIdx].broken = 1;
						}
				}
				V.set(a, b0.lin, b0.ang);
				if(dynB) V.set(b, b1.lin, b1.ang);
			}
			// this chunk's slot is overwritten by a later bulk copy; its records' impulses
			// are read by one
			fenceProxyAsync();
			fenceProxyAsyncGlobal();
			groupSync(barId, nt);
		}
		if(posIter)
		{
			for(uint32_t i = gtid; i < n; i += nt)
			{
				tgs::BodyVel v;
				v.lin = V.lin(i); v.ang = V.ang(i); v.dLin = V.dLin(i); v.dAng = V.dAng(i);
				tgs::integrateStep(v, tx[i], stepDt);
				V.setDelta(i, v.dLin, v.dAng);
			}
			elapsed += stepDt;
			groupSync(barId, nt);
		}
	}
	for(uint32_t i = gtid; i < n; i += nt)
	{
		tgs::BodyVel v;
		v.lin = V.lin(i); v.ang = V.ang(i); v.dLin = V.dLin(i); v.dAng = V.dAng(i);
		Tr p = pose[i];
		V3 wv;
		tgs::finalizeBody(v, tx[i], p, wv);
		tgs::RigidBody& rb = w.bodies[sc.bodyStart + i];
		rb.linVel[0] = v.lin.x; rb.linVel[1] = v.lin.y; rb.linVel[2] = v.lin.z;
		rb.angVel[0] = wv.x; rb.angVel[1] = wv.y; rb.angVel[2] = wv.z;
		rb.q[0] = p.q.x; rb.q[1] = p.q.y; rb.q[2] = p.q.z; rb.q[3] = p.q.w;
		rb.p[0] = p.p.x; rb.p[1] = p.p.y; rb.p[2] = p.p.z;
	}
	// parities after this scene's fills (slot 0: ceil(nSeq / 2), slot 1: floor)
	groupSync(barId, nt);
	if(gtid == 0)
	{
		phase[0] = ph0 ^ (((nSeq + 1) >> 1) & 1u);
		phase[1] = ph1 ^ ((nSeq >> 1) & 1u);
	}
	return true;
}

// Per-group state of the resident solve kept in static shared memory.
struct ResGroupState
{
	unsigned long long* bar;   // the group's bulk-copy barrier
	uint32_t* phase;           // parity of the barrier phase the group waits for next
	uint32_t* word;            // broadcast word
	uint32_t* scratch;         // one word per warp of the group
};

// One scene on one group's slice: partition ends, row offsets, the rows (bulk
// copies, one per constraint, completing on the group's barrier) and the body
// velocities go on chip, then the iterations run there.  Returns false when a
// bulk copy did not complete within the wait limit (the scene is flagged
// ST_STAGE_TIMEOUT and the group stops).
__device__ __forceinline__ bool solveResidentScene(const WorldDev& w, uint32_t sid, const StepParams& sp, unsigned char* slice, uint32_t sliceBytes,
                                   const ResGroupState& gs, uint32_t gtid, uint32_t nt, uint32_t barId)
{
	const SceneDesc sc = w.scenes[sid];
	const uint32_t nbPart = w.nbPartitions[sid];
	const uint32_t ncAll = w.nbConstraints[sid];
	if(nbPart || !ncAll)   // batching overflowed: the scene is left unchanged
	{
		const uint32_t nc = nbPart ? ncAll : 0u;
		const uint32_t nTot = sc.nbBodies + sc.nbStatics;
		uint32_t* ends = reinterpret_cast<uint32_t*>(slice);
		uint16_t* off = reinterpret_cast<uint16_t*>(slice + RES_HEADER);
		const uint32_t offBytes = align16(2 * nc), velBytes = align16(48 * nTot);
		V3* velBase = reinterpret_cast<V3*>(slice + RES_HEADER + offBytes);
		unsigned char* rows = slice + RES_HEADER + offBytes + velBytes;
		// this thread's run of constraints and the offset of its first row chunk
		const uint32_t per = (nc + nt - 1) / nt;
		const uint32_t r0 = min(gtid * per, nc), r1 = min(r0 + per, nc);
		const uint8_t* chunks = w.recChunks + sc.pairStart;
		uint32_t runChunks = 0;
		for(uint32_t r = r0; r < r1; r++) runChunks += chunks[r];
		uint32_t total = 0;
		const uint32_t first = groupPrefix(runChunks, gs.scratch, gtid, nt, barId, total);
		const bool velOnChip = RES_HEADER + offBytes + velBytes <= sliceBytes;
		const bool rowsOnChip = velOnChip && RES_HEADER + offBytes + velBytes + 16u * total <= sliceBytes;
		// streamed rows: a two-slot ring after the chunk table
		const uint32_t tableOff = RES_HEADER + offBytes + velBytes, ringOff = tableOff + align16(RES_TABLE);
		const uint32_t slotBytes = ringOff < sliceBytes ? ((sliceBytes - ringOff) / 2u) & ~15u : 0u;
		bool stream = sp.resStream && velOnChip && !rowsOnChip && nt >= 64 && nbPart > 0 && total > 0 && total <= 65535u &&
		              slotBytes >= RES_MIN_SLOT;
		// the slice was last read by generic loads (previous scene): order them
		// before the bulk copies that overwrite it
		fenceProxyAsync();
		for(uint32_t p = gtid; p < nbPart; p += nt) ends[p] = w.partEnds[size_t(sid) * MAX_PARTITIONS + p];
		const bool staging = rowsOnChip && total > 0;
		if(staging)
		{
			if(gtid == 0) mbarArriveExpectTx(gs.bar, 16u * total);
			groupSync(barId, nt);
			uint32_t o = first;
			for(uint32_t r = r0; r < r1; r++)
			{
				const uint32_t c = chunks[r];
				off[r] = uint16_t(o);
				bulkCopyToShared(rows + 16u * o, w.recs + sc.pairStart + r, 16u * c, gs.bar);
				o += c;
			}
		}
		uint32_t* chunkFirst = reinterpret_cast<uint32_t*>(slice + tableOff);
		uint32_t* partChunk = chunkFirst + RES_MAX_CHUNKS + 1;
		uint32_t nChunks = 0;
		if(stream)
		{
			uint32_t o = first;
			for(uint32_t r = r0; r < r1; r++)
			{
				off[r] = uint16_t(o);
				o += chunks[r];
			}
			groupSync(barId, nt);
			// chunk k of partition p: its constraints whose rows start in
			// [k, k + 1) * capU units after the partition's first row (at most a slot)
			const uint32_t capU = slotBytes / 16u - RES_RECORD_UNITS;
			if(gtid < 32)
			{
				uint32_t carry = 0;
				for(uint32_t p0 = 0; p0 < nbPart; p0 += 32)
				{
					const uint32_t p = p0 + gtid;
					uint32_t cnt = 0;
					if(p < nbPart)
					{
						const uint32_t b = p ? ends[p - 1] : 0u, e = ends[p];
						if(e > b) cnt = uint32_t(off[e - 1] - off[b]) / capU + 1u;
					}
					uint32_t incl = cnt;
					for(int d = 1; d < 32; d <<= 1)
					{
						const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
						if(gtid >= uint32_t(d)) incl += t;
					}
					if(p < nbPart) partChunk[p] = carry + incl - cnt;
					carry += __shfl_sync(0xffffffffu, incl, 31);
				}
				if(gtid == 0) partChunk[nbPart] = carry;
			}
			groupSync(barId, nt);
			nChunks = partChunk[nbPart];
			stream = nChunks <= RES_MAX_CHUNKS;
			if(stream)
			{
				for(uint32_t r = gtid; r < nc; r += nt)
				{
					uint32_t lo = 0, hi = nbPart - 1;   // partition of r: first p with ends[p] > r
					while(lo < hi)
					{
						const uint32_t mid = (lo + hi) >> 1;
						if(ends[mid] > r) hi = mid;
						else lo = mid + 1;
					}
					const uint32_t b = lo ? ends[lo - 1] : 0u;
					const uint32_t k = uint32_t(off[r] - off[b]) / capU;
					if(r == b || k != uint32_t(off[r - 1] - off[b]) / capU) chunkFirst[partChunk[lo] + k] = r;
				}
				if(gtid == 0) chunkFirst[nChunks] = nc;
			}
			groupSync(barId, nt);
		}
		const ResVel rv = {velBase, velBase + nTot, velBase + 2 * nTot, velBase + 3 * nTot};
		if(velOnChip)
		{
			const tgs::BodyVel* vel = w.vel + sc.solverStart;
			for(uint32_t i = gtid; i < nTot; i += nt)
			{
				const tgs::BodyVel v = vel[i];
				rv.set(i, v.lin, v.ang);
				rv.setDelta(i, v.dLin, v.dAng);
			}
		}
		if(staging)
		{
			const uint32_t parity = *gs.phase;
			bool done = false;
			for(uint32_t k = 0; k < STAGE_WAIT_LIMIT && !done; k++) done = mbarTryWait(gs.bar, parity);
			const bool allDone = __all_sync(0xffffffffu, done);
			if(!allDone && (gtid & 31) == 0) atomicOr(gs.word, 1u);
			groupSync(barId, nt);
			if(*gs.word)
			{
				// a copy is lost: flag the scene, give the copies in flight a last bounded
				// wait (they write into this slice), and stop this group
				if(gtid == 0) atomicOr(&w.status[sid], ST_STAGE_TIMEOUT);
				for(uint32_t k = 0; k < STAGE_WAIT_LIMIT && !done; k++) done = mbarTryWait(gs.bar, parity);
				return false;
			}
			groupSync(barId, nt);
			if(gtid == 0) *gs.phase = parity ^ 1u;
		}
		groupSync(barId, nt);
		if(rowsOnChip) residentIterate<true>(w, sc, sid, sp, ends, nbPart, off, rows, rv, gtid, nt, barId);
		else if(stream)
		{
			if(!residentIterateStreamed(w, sc, sid, sp, ends, nbPart, off, total, chunkFirst, nChunks, slice + ringOff, slotBytes, rv, gtid, nt,
			                            barId, gs.bar, gs.phase, gs.word))
				return false;
		}
		else if(velOnChip) residentIterate<false>(w, sc, sid, sp, ends, nbPart, off, rows, rv, gtid, nt, barId);
		else residentIterate<false>(w, sc, sid, sp, ends, nbPart, off, rows, ResHbmVel{w.vel + sc.solverStart}, gtid, nt, barId);
	}
	groupSync(barId, nt);
	if(sp.persistent && gtid == 0) w.sceneParity[sid] ^= 1u;
	return true;
}

// The resident solve: persistent, one block per SM.  Level by level (largest
// footprints first) the block's groups take scenes from the level's list;
// a group that finds its level's list empty splits into the next level's
// groups, which go on without waiting for the rest of the block.
__global__ void __launch_bounds__(RES_WARPS * 32, 1) solveResidentKernel(WorldDev w, StepParams sp)
{
	extern __shared__ __align__(128) unsigned char resSmem[];
	__shared__ __align__(8) unsigned long long bar[RES_WARPS];
	__shared__ uint32_t phase[RES_WARPS], word[RES_WARPS], scratch[RES_WARPS];
	const uint32_t warp = threadIdx.x >> 5;
	if(threadIdx.x < RES_WARPS)
	{
		mbarInit(&bar[threadIdx.x], 1);
		phase[threadIdx.x] = 0;
		word[threadIdx.x] = 0;
	}
	asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
	__syncthreads();
	for(uint32_t level = 0; level < RES_LEVELS; level++)
	{
		const uint32_t gw = RES_WARPS >> level, group = warp / gw, first = group * gw;
		const uint32_t nt = gw * 32, gtid = threadIdx.x - first * 32;
		// named barrier of the group: 2^level + group (1 .. 2 * RES_WARPS - 1); single warps use __syncwarp
		const uint32_t barId = nt > 32 ? (1u << level) + group : 0u;
		const uint32_t sliceBytes = sp.resBytes >> level;
		unsigned char* slice = resSmem + size_t(group) * sliceBytes;
		const ResGroupState gs = {&bar[first], &phase[first], &word[first], &scratch[first]};
		const uint32_t count = w.workCounter[WC_RES_COUNT + level];
		for(;;)
		{
			if(gtid == 0) *gs.word = atomicAdd(&w.workCounter[WC_RES_NEXT + level], 1u);
			groupSync(barId, nt);
			const uint32_t idx = *gs.word;
			groupSync(barId, nt);
			if(idx >= count) break;
			if(gtid == 0) *gs.word = 0;   // the timeout vote of this scene
			groupSync(barId, nt);
			if(!solveResidentScene(w, w.resList[size_t(level) * w.resCap + idx], sp, slice, sliceBytes, gs, gtid, nt, barId)) return;
			groupSync(barId, nt);
		}
	}
}

// Totals over all scenes after a step: pairs, pairs with contacts, contacts.
// Totals of the last step: pairs, pairs with contacts, contacts, bytes of packed
// constraint rows (what every solver iteration reads).
__global__ void statsKernel(const SceneDesc* __restrict__ scenes, uint32_t nbScenes, const uint32_t* __restrict__ pairCount,
                            const uint32_t* __restrict__ contactCount, const uint32_t* __restrict__ nbConstraints,
                            const uint32_t* __restrict__ nbPartitions, const uint8_t* __restrict__ recChunks, unsigned long long* __restrict__ out)
{
	const uint32_t sid = blockIdx.x;
	if(sid >= nbScenes) return;
	const SceneDesc sc = scenes[sid];
	const uint32_t count = pairCount[sid];
	const uint32_t nc = nbPartitions[sid] ? nbConstraints[sid] : 0;
	unsigned long long withContacts = 0, contacts = 0, rowBytes = 0;
	for(uint32_t k = threadIdx.x; k < count; k += blockDim.x)
	{
		const uint32_t c = contactCount[sc.pairStart + k];
		withContacts += c ? 1 : 0;
		contacts += c;
	}
	for(uint32_t r = threadIdx.x; r < nc; r += blockDim.x) rowBytes += 16ull * recChunks[sc.pairStart + r];
	for(int o = 16; o > 0; o >>= 1)
	{
		withContacts += __shfl_down_sync(0xffffffffu, withContacts, o);
		contacts += __shfl_down_sync(0xffffffffu, contacts, o);
		rowBytes += __shfl_down_sync(0xffffffffu, rowBytes, o);
	}
	if((threadIdx.x & 31) == 0)
	{
		atomicAdd(&out[1], withContacts);
		atomicAdd(&out[2], contacts);
		atomicAdd(&out[3], rowBytes);
	}
	if(threadIdx.x == 0) atomicAdd(&out[0], static_cast<unsigned long long>(count));
}
} // namespace world

// Host-side world: scene table, resident state, scratch, graph.
struct World
{
	cudaStream_t stream = 0;
	cudaStream_t sideStream = 0;   // block-per-scene kernels run beside the warp-per-scene ones
	int streamPriority = 0;        // CUDA stream priority of the world's streams (set before create)
	cudaEvent_t forkEv[4] = {}, joinEv[4] = {};
	cudaGraphExec_t graphExec = nullptr;
	uint32_t graphSteps = 0;
	world::StepParams params;
	std::vector<world::SceneDesc> hScenes;
	uint32_t nbScenes = 0, nbBodies = 0, nbStatics = 0, nbSolver = 0, nbKeys = 0, nbPairSlots = 0;
	uint32_t gridBlocks = 0, gridBatch = 0, gridPrep = 0, gridSolve[world::SOLVE_VARIANTS] = {}, gridNp[world::NB_KINDS] = {};
	uint32_t gridBpBig = 0, gridBatchBig = 0, gridSolveBig = 0, gridOrder = 0, gridPrepOrder = 0, gridRes = 0;
	uint32_t maxSolverBodies = 0;   // largest scene (bodies + statics) a slot can hold
	// persistent blocks per SM of the row preparation and of the capsule-box and
	// box-box narrowphase kernels (0: as many as fit).  Their threads keep large
	// per-thread working sets in local memory (friction correlation, GJK/EPA), and
	// fewer threads in flight keep that memory in L1 / L2 instead of HBM.
	uint32_t sms = 0, prepPerSm = 0, npHeavyPerSm = 0;
	uint32_t prepGrid() const { return prepPerSm ? std::min(gridPrep, sms * prepPerSm) : gridPrep; }
	uint32_t npGrid(uint32_t k) const { return (k == 7 || k == 8) && npHeavyPerSm ? std::min(gridNp[k], sms * npHeavyPerSm) : gridNp[k]; }
	uint32_t pairsPerBody = 0;
	// scenes above this many solver bodies run one block per scene (warp per scene below)
	static constexpr uint32_t DEFAULT_LARGE_BODIES = 512;
	static constexpr uint32_t DEFAULT_RES_STREAM = 1;   // streamed-row levels of the resident solve
	static constexpr uint32_t BIG_THREADS = world::BIG_WARPS * 32;
	static constexpr uint32_t RES_THREADS = world::RES_WARPS * 32;
	bool resident() const { return params.solveVariant == world::RESIDENT_VARIANT; }
	bool launchLarge() const { return maxSolverBodies > params.largeBodies; }
	DevBuf<world::SceneDesc> scenes;
	DevBuf<uint32_t> typeQueueSorted;
	DevBuf<uint32_t> typeQueue, slotScene, nbConstraints, nbPartitions, prepQueue, activeCount;
	DevBuf<uint32_t> prepQueueSorted;
	DevBuf<uint8_t> prepClass;
	DevBuf<uint8_t> recChunks;
	DevBuf<uint32_t> workOrder, workCounter, pairs, pairCount, contactCount, ordered, consList, tag, progress, maxNormal, maxStatic,
	    staticProgress, partEnds, status;
	DevBuf<tgs::RigidBody> bodies;
	DevBuf<int> types, staticTypes;
	DevBuf<float4> geoms, staticGeoms, contacts;
	DevBuf<float> friction, staticPose, aabb;
	DevBuf<unsigned long long> keys, stats;
	DevBuf<uint32_t> identity;
	DevBuf<tgs::ConstraintRecord> recs;
	DevBuf<uint32_t> pairsPrev, pairCountPrev, prevSlot, sceneParity;
	DevBuf<np::ManifoldRecord> manifolds[2];
	DevBuf<tgs::FrictionState> frictionState[2];
	DevBuf<unsigned long long> sceneAcc;
	DevBuf<uint32_t> resList;
	DevBuf<tgs::BodyVel> vel;
	DevBuf<tgs::BodyTx> tx;
	DevBuf<tgs::BodyData> data;
	DevBuf<Tr> pose;
	HostBuf<tgs::RigidBody> hStage;
	size_t deviceBytes = 0;

	static uint32_t pow2(uint32_t x) { uint32_t p = 1; while(p < x) p <<= 1; return p; }
	// work counters of the broadphase and solve kernels, then the per-kind pair counts
	static constexpr uint32_t COUNTERS = world::NB_WORK_COUNTERS;
	static_assert(world::WC_RES_COUNT == 8 + world::NB_KINDS + 4, "resident-solve counters follow the pair-kind and path counters");
	// broadphase, one narrowphase kernel per pair kind, batching, row preparation, solve
	static constexpr uint32_t KERNELS_PER_STEP = 4 + world::NB_KINDS;

	world::WorldDev dev()
	{
		world::WorldDev w;
		w.scenes = scenes.ptr; w.workOrder = workOrder.ptr; w.nbActive = activeCount.ptr; w.workCounter = workCounter.ptr;
		w.bodies = bodies.ptr; w.types = types.ptr; w.geoms = geoms.ptr; w.friction = friction.ptr;
		w.staticPose = staticPose.ptr; w.staticTypes = staticTypes.ptr; w.staticGeoms = staticGeoms.ptr;
		w.aabb = aabb.ptr; w.keys = keys.ptr; w.pairs = pairs.ptr; w.pairCount = pairCount.ptr; w.contacts = contacts.ptr;
		w.contactCount = contactCount.ptr; w.ordered = ordered.ptr; w.consList = consList.ptr; w.tag = tag.ptr; w.recs = recs.ptr;
		w.vel = vel.ptr; w.tx = tx.ptr; w.data = data.ptr; w.pose = pose.ptr; w.progress = progress.ptr; w.maxNormal = maxNormal.ptr;
		w.maxStatic = maxStatic.ptr; w.staticProgress = staticProgress.ptr; w.partEnds = partEnds.ptr; w.status = status.ptr;
		w.typeCount = workCounter.ptr + 8; w.pathCount = workCounter.ptr + 8 + world::NB_KINDS; w.typeQueueSorted = typeQueueSorted.ptr;
		w.typeQueue = typeQueue.ptr; w.queueCap = nbPairSlots; w.slotScene = slotScene.ptr;
		w.nbConstraints = nbConstraints.ptr; w.nbPartitions = nbPartitions.ptr; w.prepQueue = prepQueue.ptr; w.prepQueueSorted = prepQueueSorted.ptr; w.prepClass = prepClass.ptr; w.recChunks = recChunks.ptr;
		w.pairsPrev = pairsPrev.ptr; w.pairCountPrev = pairCountPrev.ptr; w.prevSlot = prevSlot.ptr; w.sceneParity = sceneParity.ptr;
		for(int k = 0; k < 2; k++) { w.manifolds[k] = manifolds[k].ptr; w.frictionState[k] = frictionState[k].ptr; }
		w.sceneAcc = sceneAcc.ptr; w.resList = resList.ptr; w.resCap = nbScenes;
		return w;
	}

	int create(uint32_t S, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, const void* rigid, const int* typesIn,
	           const float* geomsIn, const float* frictionIn, const float* staticPoseIn, const int* staticTypesIn, const float* staticGeomsIn,
	           uint32_t pairsPerBodyIn, const world::StepParams& sp)
	{
		params = sp;
		pairsPerBody = pairsPerBodyIn;
		nbScenes = S;
		hScenes.resize(S);
		uint32_t b = 0, st = 0, key = 0, pair = 0;
		for(uint32_t s = 0; s < S; s++)
		{
			world::SceneDesc& d = hScenes[s];
			if(sceneBodyCount[s] == 0 || sceneBodyCount[s] + sceneStaticCount[s] > 65535u) return GBPX_ERR_INVALID;
			d.bodyStart = b; d.nbBodies = sceneBodyCount[s];
			d.staticStart = st; d.nbStatics = sceneStaticCount[s];
			d.solverStart = b + st;
			d.keyStart = key; d.keyCap = pow2(d.nbBodies);
			d.pairStart = pair; d.pairCap = pow2(d.nbBodies * pairsPerBody + d.nbBodies * d.nbStatics);
			if(uint64_t(pair) + d.pairCap >= (1ull << 31)) return GBPX_ERR_CAPACITY;   // pair slots are 31-bit queue entries
			b += d.nbBodies; st += d.nbStatics; key += d.keyCap; pair += d.pairCap;
		}
		nbBodies = b; nbStatics = st; nbSolver = b + st; nbKeys = key; nbPairSlots = pair;
		for(const world::SceneDesc& d : hScenes) maxSolverBodies = std::max(maxSolverBodies, d.nbBodies + d.nbStatics);
		std::vector<uint32_t> order(S);
		std::iota(order.begin(), order.end(), 0u);
		std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return hScenes[x].nbBodies > hScenes[y].nbBodies; });
		GBPX_CUDA_TRY(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, streamPriority));
		GBPX_CUDA_TRY(cudaStreamCreateWithPriority(&sideStream, cudaStreamNonBlocking, streamPriority));
		for(int k = 0; k < 4; k++)
		{
			GBPX_CUDA_TRY(cudaEventCreateWithFlags(&forkEv[k], cudaEventDisableTiming));
			GBPX_CUDA_TRY(cudaEventCreateWithFlags(&joinEv[k], cudaEventDisableTiming));
		}
		if(scenes.reserve(S) || workOrder.reserve(S) || workCounter.reserve(COUNTERS) || typeQueue.reserve(size_t(world::NB_KINDS) * pair) || slotScene.reserve(pair) || activeCount.reserve(2) || recChunks.reserve(pair) || nbConstraints.reserve(S) || nbPartitions.reserve(S) || prepQueue.reserve(pair) || prepQueueSorted.reserve(pair) || prepClass.reserve(pair) || bodies.reserve(b) || types.reserve(b) || geoms.reserve(b) ||
		   friction.reserve(b) || staticPose.reserve(7 * size_t(st) + 1) || staticTypes.reserve(st + 1) || staticGeoms.reserve(st + 1) ||
		   aabb.reserve(6 * size_t(b)) || keys.reserve(key) || pairs.reserve(pair) || pairCount.reserve(S) || contacts.reserve(8 * size_t(pair)) ||
		   contactCount.reserve(pair) || ordered.reserve(pair) || consList.reserve(pair) || tag.reserve(pair) || recs.reserve(pair) ||
		   vel.reserve(nbSolver) || tx.reserve(nbSolver) || data.reserve(nbSolver) || pose.reserve(nbSolver) || progress.reserve(nbSolver) ||
		   maxNormal.reserve(nbSolver) || maxStatic.reserve(nbSolver) || staticProgress.reserve(nbSolver) ||
		   partEnds.reserve(size_t(S) * world::MAX_PARTITIONS) || status.reserve(S) || hStage.reserve(b) || stats.reserve(4) ||
		   identity.reserve(S) || pairCountPrev.reserve(S) || sceneParity.reserve(S) || sceneAcc.reserve(S) ||
		   resList.reserve(size_t(world::RES_LEVELS) * S))
			return GBPX_ERR_NOMEM;
		if(sp.persistent &&
		   (pairsPrev.reserve(pair) || prevSlot.reserve(pair) || manifolds[0].reserve(pair) || manifolds[1].reserve(pair) ||
		    frictionState[0].reserve(pair) || frictionState[1].reserve(pair) || typeQueueSorted.reserve(2 * size_t(pair))))
			return GBPX_ERR_NOMEM;
		deviceBytes = size_t(pair) * (4 + 128 + 4 * 4 + 4 + 4 * world::NB_KINDS + sizeof(tgs::ConstraintRecord)) + size_t(b) * (96 + 4 + 16 + 4 + 24) +
		              size_t(nbSolver) * (sizeof(tgs::BodyVel) + sizeof(tgs::BodyTx) + sizeof(tgs::BodyData) + sizeof(Tr) + 16) + size_t(key) * 8;
		if(sp.persistent) deviceBytes += size_t(pair) * (8 + 2 * (sizeof(np::ManifoldRecord) + sizeof(tgs::FrictionState)));
		cudaStream_t s = stream;
		GBPX_CUDA_TRY(cudaMemcpyAsync(scenes.ptr, hScenes.data(), S * sizeof(world::SceneDesc), cudaMemcpyHostToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(workOrder.ptr, order.data(), S * 4, cudaMemcpyHostToDevice, s));
		std::vector<uint32_t> owner(pair);
		for(uint32_t sc = 0; sc < S; sc++)
			std::fill(owner.begin() + hScenes[sc].pairStart, owner.begin() + hScenes[sc].pairStart + hScenes[sc].pairCap, sc);
		GBPX_CUDA_TRY(cudaMemcpyAsync(slotScene.ptr, owner.data(), size_t(pair) * 4, cudaMemcpyHostToDevice, s));
		std::vector<uint32_t> ident(S);
		std::iota(ident.begin(), ident.end(), 0u);
		GBPX_CUDA_TRY(cudaMemcpyAsync(identity.ptr, ident.data(), S * 4, cudaMemcpyHostToDevice, s));
		const uint32_t activeInit[2] = {S, 1u};   // all scenes; one scene (the unbatched path)
		GBPX_CUDA_TRY(cudaMemcpyAsync(activeCount.ptr, activeInit, 8, cudaMemcpyHostToDevice, s));
		if(!rigid)
		{
			// capacity only (serving slots): contents arrive with each admitted scene
			GBPX_CUDA_TRY(cudaMemsetAsync(bodies.ptr, 0, size_t(b) * sizeof(tgs::RigidBody), s));
			GBPX_CUDA_TRY(cudaMemsetAsync(types.ptr, 0, size_t(b) * 4, s));
			GBPX_CUDA_TRY(cudaMemsetAsync(geoms.ptr, 0, size_t(b) * 16, s));
			GBPX_CUDA_TRY(cudaMemsetAsync(friction.ptr, 0, size_t(b) * 4, s));
		}
		else
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(bodies.ptr, rigid, size_t(b) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, s));
			GBPX_CUDA_TRY(cudaMemcpyAsync(types.ptr, typesIn, size_t(b) * 4, cudaMemcpyHostToDevice, s));
			GBPX_CUDA_TRY(cudaMemcpyAsync(geoms.ptr, geomsIn, size_t(b) * 16, cudaMemcpyHostToDevice, s));
			GBPX_CUDA_TRY(cudaMemcpyAsync(friction.ptr, frictionIn, size_t(b) * 4, cudaMemcpyHostToDevice, s));
		}
		if(st && staticPoseIn)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticPose.ptr, staticPoseIn, size_t(st) * 28, cudaMemcpyHostToDevice, s));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticTypes.ptr, staticTypesIn, size_t(st) * 4, cudaMemcpyHostToDevice, s));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticGeoms.ptr, staticGeomsIn, size_t(st) * 16, cudaMemcpyHostToDevice, s));
		}
		GBPX_CUDA_TRY(cudaMemsetAsync(status.ptr, 0, S * 4, s));
		// no pair has a history yet
		GBPX_CUDA_TRY(cudaMemsetAsync(pairCount.ptr, 0, S * 4, s));
		GBPX_CUDA_TRY(cudaMemsetAsync(pairCountPrev.ptr, 0, S * 4, s));
		GBPX_CUDA_TRY(cudaMemsetAsync(sceneParity.ptr, 0, S * 4, s));
		int dev = 0, sms = 0;
		GBPX_CUDA_TRY(cudaGetDevice(&dev));
		GBPX_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::broadphaseKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bpSmemBytes(world::STAGE_WARPS))));
		GBPX_CUDA_TRY(gridFor(world::broadphaseKernel, sms, gridBlocks, bpSmemBytes(world::STAGE_WARPS)));
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::batchKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(solveSmemBytes(world::STAGE_WARPS))));
		GBPX_CUDA_TRY(gridFor(world::batchKernel, sms, gridBatch, solveSmemBytes(world::STAGE_WARPS)));
		GBPX_CUDA_TRY(gridFor(world::prepKernel, sms, gridPrep));
		this->sms = uint32_t(sms);
		for(uint32_t v = 0; v < world::SOLVE_VARIANTS; v++)
		{
			GBPX_CUDA_TRY(cudaFuncSetAttribute(solveKernels()[v], cudaFuncAttributeMaxDynamicSharedMemorySize, int(iterSmemBytes(world::SOLVE_WARPS, v))));
			GBPX_CUDA_TRY(gridFor(solveKernels()[v], sms, gridSolve[v], iterSmemBytes(world::SOLVE_WARPS, v), world::SOLVE_WARPS * 32));
		}
		for(uint32_t k = 0; k < world::NB_KINDS; k++) GBPX_CUDA_TRY(gridFor(npKernels()[k], sms, gridNp[k]));
		GBPX_CUDA_TRY(gridFor(world::orderByPathKernel, sms, gridOrder));
		GBPX_CUDA_TRY(gridFor(world::prepOrderKernel, sms, gridPrepOrder));
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::broadphaseBigKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(world::BpSmemBig))));
		GBPX_CUDA_TRY(gridFor(world::broadphaseBigKernel, sms, gridBpBig, sizeof(world::BpSmemBig), int(BIG_THREADS)));
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::batchBigKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(world::SolveSmemBig))));
		GBPX_CUDA_TRY(gridFor(world::batchBigKernel, sms, gridBatchBig, sizeof(world::SolveSmemBig), int(BIG_THREADS)));
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::solveBigKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(world::IterSmemBig))));
		GBPX_CUDA_TRY(gridFor(world::solveBigKernel, sms, gridSolveBig, sizeof(world::IterSmemBig), int(BIG_THREADS)));
		// resident solve: all the opt-in shared memory a block may have, less the
		// kernel's static part, rounded so that every level's slice stays 16-byte
		// aligned (bulk copies and float4 rows need it); one block per SM
		int optin = 0;
		GBPX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
		cudaFuncAttributes fa;
		GBPX_CUDA_TRY(cudaFuncGetAttributes(&fa, world::solveResidentKernel));
		const size_t unit = size_t(16) << (world::RES_LEVELS - 1);   // the deepest level's slice stays a multiple of 16 bytes
		params.resBytes = uint32_t((size_t(optin) - fa.sharedSizeBytes) / unit * unit);
		GBPX_CUDA_TRY(cudaFuncSetAttribute(world::solveResidentKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(params.resBytes)));
		GBPX_CUDA_TRY(gridFor(world::solveResidentKernel, sms, gridRes, params.resBytes, int(RES_THREADS)));
		GBPX_CUDA_TRY(cudaStreamSynchronize(s));
		return GBPX_OK;
	}

	typedef void (*StageKernel)(world::WorldDev, world::StepParams);
	static const StageKernel* npKernels()
	{
		static const StageKernel k[world::NB_KINDS] = {
		    world::narrowphaseKernel<0, 0>, world::narrowphaseKernel<0, 1>, world::narrowphaseKernel<0, 2>,
		    world::narrowphaseKernel<0, 3>, world::narrowphaseKernel<1, 2>, world::narrowphaseKernel<1, 3>,
		    world::narrowphaseKernel<2, 2>, world::narrowphaseKernel<2, 3>, world::narrowphaseKernel<3, 3>};
		return k;
	}
	static size_t bpSmemBytes(uint32_t warps) { return warps * sizeof(world::BpSmem); }
	static size_t solveSmemBytes(uint32_t warps) { return warps * sizeof(world::SolveSmem); }
	static size_t iterSmemBytes(uint32_t warps, uint32_t variant)
	{
		using namespace world;
		static const size_t per[SOLVE_VARIANTS] = {sizeof(IterSmemW<SOLVE_SMEM_BODIES, 0>), sizeof(IterSmemW<SOLVE_SMEM_BODIES, 16>),
		                                           sizeof(IterSmemW<SOLVE_SMEM_BODIES, RECBUF_CHUNKS>), sizeof(IterSmemW<1, 0>),
		                                           sizeof(IterSmemW<1, 16>), sizeof(IterSmemW<1, RECBUF_CHUNKS>),
		                                           sizeof(IterSmemW<SOLVE_SMEM_BODIES, MID_CHUNKS>), sizeof(IterSmemW<1, MID_CHUNKS>)};
		return warps * per[variant];
	}
	static const StageKernel* solveKernels()
	{
		using namespace world;
		static const StageKernel k[SOLVE_VARIANTS] = {solveKernel<SOLVE_SMEM_BODIES, 0>, solveKernel<SOLVE_SMEM_BODIES, 16>,
		                                              solveKernel<SOLVE_SMEM_BODIES, RECBUF_CHUNKS>, solveKernel<1, 0>, solveKernel<1, 16>,
		                                              solveKernel<1, RECBUF_CHUNKS>, solveKernel<SOLVE_SMEM_BODIES, MID_CHUNKS>,
		                                              solveKernel<1, MID_CHUNKS>};
		return k;
	}
	// persistent grid: every SM filled to the kernel's occupancy at 128 threads per block
	static cudaError_t gridFor(StageKernel k, int sms, uint32_t& grid, size_t smem = 0, int threads = 128)
	{
		int perSm = 0;
		const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, threads, smem);
		grid = uint32_t(sms * (perSm > 0 ? perSm : 1));
		return e;
	}

	// One step: clear the counters, broadphase, one narrowphase kernel per
	// pair kind, solve.  `plainScene` < nbScenes steps that scene alone with
	// single-warp scene stages (the unbatched comparison point).
	int launchStep(uint32_t plainScene = ~0u)
	{
		world::WorldDev w = dev();
		const uint32_t sv = params.solveVariant;
		uint32_t gBp = gridBlocks, gBatch = gridBatch, gPrep = prepGrid(), gSolve = gridSolve[sv], threads = 128;
		const bool plain = plainScene < nbScenes;
		if(plain)
		{
			w.workOrder = identity.ptr + plainScene;
			w.nbActive = activeCount.ptr + 1;
			gBp = gBatch = gSolve = 1;
			gPrep = std::min(gridPrep, 8u);
			threads = 32;
		}
		const bool big = launchLarge();
		// block-per-scene kernels run on the side stream, concurrently with the
		// warp-per-scene ones (separate work counters); joined before the next stage
		auto fork = [&](int k) -> cudaError_t {
			cudaError_t e = cudaEventRecord(forkEv[k], stream);
			return e != cudaSuccess ? e : cudaStreamWaitEvent(sideStream, forkEv[k], 0);
		};
		auto join = [&](int k) -> cudaError_t {
			cudaError_t e = cudaEventRecord(joinEv[k], sideStream);
			return e != cudaSuccess ? e : cudaStreamWaitEvent(stream, joinEv[k], 0);
		};
		const cudaStream_t bigStream = plain ? stream : sideStream;
		Zone zone(plain ? "gbpx::world::launchPlainStep" : "gbpx::world::launchStep");
		GBPX_CUDA_TRY(cudaMemsetAsync(workCounter.ptr, 0, COUNTERS * 4, stream));
		if(big && !plain) GBPX_CUDA_TRY(fork(0));
		world::broadphaseKernel<<<gBp, threads, bpSmemBytes(threads / 32), stream>>>(w, params);
		if(big)
		{
			world::broadphaseBigKernel<<<plain ? 1u : gridBpBig, BIG_THREADS, sizeof(world::BpSmemBig), bigStream>>>(w, params);
			if(!plain) GBPX_CUDA_TRY(join(0));
		}
		// the pair kinds write disjoint slots: capsule-box and box-box (the long
		// kernels) run on the side stream beside the seven other kinds
		if(!plain) GBPX_CUDA_TRY(fork(3));
		const cudaStream_t heavyStream = plain ? stream : sideStream;
		for(uint32_t k = 7; k < world::NB_KINDS; k++)
		{
			if(k == 7 && params.persistent) world::orderByPathKernel<<<plain ? std::min(gridOrder, 8u) : gridOrder, 128, 0, heavyStream>>>(w, params);
			npKernels()[k]<<<plain ? std::min(gridNp[k], 8u) : npGrid(k), 128, 0, heavyStream>>>(w, params);
		}
		for(uint32_t k = 0; k < 7; k++) npKernels()[k]<<<plain ? std::min(gridNp[k], 8u) : npGrid(k), 128, 0, stream>>>(w, params);
		if(!plain) GBPX_CUDA_TRY(join(3));
		if(big && !plain) GBPX_CUDA_TRY(fork(1));
		world::batchKernel<<<gBatch, threads, solveSmemBytes(threads / 32), stream>>>(w, params);
		if(big)
		{
			world::batchBigKernel<<<plain ? 1u : gridBatchBig, BIG_THREADS, sizeof(world::SolveSmemBig), bigStream>>>(w, params);
			if(!plain) GBPX_CUDA_TRY(join(1));
		}
		world::prepOrderKernel<<<plain ? std::min(gridPrepOrder, 8u) : gridPrepOrder, 128, 0, stream>>>(w, params);
		world::prepKernel<<<gPrep, 128, 0, stream>>>(w, params);
		if(resident())
			// every scene, large or small, in one launch
			world::solveResidentKernel<<<plain ? 1u : gridRes, RES_THREADS, params.resBytes, stream>>>(w, params);
		else
		{
			const uint32_t solveThreads = plain ? 32 : world::SOLVE_WARPS * 32;
			if(big && !plain) GBPX_CUDA_TRY(fork(2));
			solveKernels()[sv]<<<gSolve, solveThreads, iterSmemBytes(solveThreads / 32, sv), stream>>>(w, params);
			if(big)
			{
				world::solveBigKernel<<<plain ? 1u : gridSolveBig, BIG_THREADS, sizeof(world::IterSmemBig), bigStream>>>(w, params);
				if(!plain) GBPX_CUDA_TRY(join(2));
			}
		}
		GBPX_CUDA_TRY(cudaGetLastError());
		return GBPX_OK;
	}

	// Captures `steps` consecutive steps into one CUDA graph (replayed by step()).
	int capture(uint32_t steps)
	{
		if(graphExec) { cudaGraphExecDestroy(graphExec); graphExec = nullptr; }
		cudaGraph_t graph;
		GBPX_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
		for(uint32_t i = 0; i < steps; i++)
		{
			const int rc = launchStep();
			if(rc) { cudaStreamEndCapture(stream, &graph); return rc; }
		}
		GBPX_CUDA_TRY(cudaStreamEndCapture(stream, &graph));
		GBPX_CUDA_TRY(cudaGraphInstantiate(&graphExec, graph, 0));
		GBPX_CUDA_TRY(cudaGraphDestroy(graph));
		graphSteps = steps;
		return GBPX_OK;
	}

	int step(uint32_t steps, bool useGraph)
	{
		if(useGraph)
		{
			if(!graphExec || graphSteps != 1)
			{
				const int rc = capture(1);
				if(rc) return rc;
			}
			for(uint32_t i = 0; i < steps; i++) GBPX_CUDA_TRY(cudaGraphLaunch(graphExec, stream));
		}
		else
			for(uint32_t i = 0; i < steps; i++)
			{
				const int rc = launchStep();
				if(rc) return rc;
			}
		return GBPX_OK;
	}

	int timeStages(uint32_t steps, float* outMs)
	{
		const uint32_t K = KERNELS_PER_STEP;
		std::vector<cudaEvent_t> ev(K + 1, nullptr);
		for(auto& e : ev) GBPX_CUDA_TRY(cudaEventCreate(&e));
		std::vector<double> acc(K, 0.0);
		const world::WorldDev w = dev();
		const bool big = launchLarge();
		int rc = GBPX_OK;
		for(uint32_t s = 0; s < steps && rc == GBPX_OK; s++)
		{
			GBPX_CUDA_TRY(cudaMemsetAsync(workCounter.ptr, 0, COUNTERS * 4, stream));
			uint32_t k = 0;
			GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			world::broadphaseKernel<<<gridBlocks, 128, bpSmemBytes(world::STAGE_WARPS), stream>>>(w, params);
			if(big) world::broadphaseBigKernel<<<gridBpBig, BIG_THREADS, sizeof(world::BpSmemBig), stream>>>(w, params);
			GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			for(uint32_t t = 0; t < world::NB_KINDS; t++)
			{
				if(t == 7 && params.persistent) world::orderByPathKernel<<<gridOrder, 128, 0, stream>>>(w, params);
				npKernels()[t]<<<npGrid(t), 128, 0, stream>>>(w, params);
				GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			}
			world::batchKernel<<<gridBatch, 128, solveSmemBytes(world::STAGE_WARPS), stream>>>(w, params);
			if(big) world::batchBigKernel<<<gridBatchBig, BIG_THREADS, sizeof(world::SolveSmemBig), stream>>>(w, params);
			GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			world::prepOrderKernel<<<gridPrepOrder, 128, 0, stream>>>(w, params);
			world::prepKernel<<<prepGrid(), 128, 0, stream>>>(w, params);
			GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			if(resident()) world::solveResidentKernel<<<gridRes, RES_THREADS, params.resBytes, stream>>>(w, params);
			else
			{
				solveKernels()[params.solveVariant]<<<gridSolve[params.solveVariant], world::SOLVE_WARPS * 32,
				                                      iterSmemBytes(world::SOLVE_WARPS, params.solveVariant), stream>>>(w, params);
				if(big) world::solveBigKernel<<<gridSolveBig, BIG_THREADS, sizeof(world::IterSmemBig), stream>>>(w, params);
			}
			GBPX_CUDA_TRY(cudaEventRecord(ev[k++], stream));
			GBPX_CUDA_TRY(cudaGetLastError());
			GBPX_CUDA_TRY(cudaEventSynchronize(ev[K]));
			for(uint32_t i = 0; i < K; i++)
			{
				float ms = 0.0f;
				GBPX_CUDA_TRY(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
				acc[i] += ms;
			}
		}
		for(uint32_t i = 0; i < K; i++) outMs[i] = float(acc[i] / steps);
		for(auto& e : ev) cudaEventDestroy(e);
		return rc;
	}

	// One scene per launch sequence: no batching across scenes and no graph; pair
	// state is kept or not as params.persistent says (the comparison point of the
	// batched step).
	int stepPlain(uint32_t first, uint32_t count)
	{
		for(uint32_t s = first; s < first + count && s < nbScenes; s++)
		{
			const int rc = launchStep(s);
			if(rc) return rc;
		}
		return GBPX_OK;
	}

	// Places a scene into slot `slot` (capacity fixed at creation): its bodies,
	// shapes and statics are copied in and the slot's live counts updated, in
	// stream order with the steps.
	int admit(uint32_t slot, uint32_t nb, const void* rigid, const int* typesIn, const float* geomsIn, const float* frictionIn, uint32_t ns,
	          const float* staticPoseIn, const int* staticTypesIn, const float* staticGeomsIn)
	{
		world::SceneDesc& d = hScenes[slot];
		const uint32_t b = d.bodyStart, st = d.staticStart;
		GBPX_CUDA_TRY(cudaMemcpyAsync(bodies.ptr + b, rigid, size_t(nb) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(types.ptr + b, typesIn, size_t(nb) * 4, cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(geoms.ptr + b, geomsIn, size_t(nb) * 16, cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(friction.ptr + b, frictionIn, size_t(nb) * 4, cudaMemcpyHostToDevice, stream));
		if(ns)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticPose.ptr + 7 * size_t(st), staticPoseIn, size_t(ns) * 28, cudaMemcpyHostToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticTypes.ptr + st, staticTypesIn, size_t(ns) * 4, cudaMemcpyHostToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticGeoms.ptr + st, staticGeomsIn, size_t(ns) * 16, cudaMemcpyHostToDevice, stream));
		}
		d.nbBodies = nb;
		d.nbStatics = ns;
		GBPX_CUDA_TRY(cudaMemcpyAsync(scenes.ptr + slot, &d, sizeof(d), cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(status.ptr + slot, 0, 4, stream));
		// an admitted scene starts without pair history
		GBPX_CUDA_TRY(cudaMemsetAsync(pairCount.ptr + slot, 0, 4, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(pairCountPrev.ptr + slot, 0, 4, stream));
		return GBPX_OK;
	}

	// Snapshot of a scene between steps (this library's byte layout): a header
	// (magic, version, bodies, statics, pairs, whether pair state follows), the
	// bodies (PxRigidBodyData), shapes, statics and, in persistent mode, the
	// sorted pair list with each pair's contact manifold and friction patches as
	// the last step left them (the buffer sceneParity names).  Restoring it into
	// a slot of enough capacity continues the scene with the same results.
	struct SnapshotHeader { uint32_t magic, version, nbBodies, nbStatics, nbPairs, pairState, pad[2]; };
	static constexpr uint32_t SNAPSHOT_MAGIC = 0x53535847u;   // "GXSS"
	static size_t snapshotBytes(uint32_t nb, uint32_t ns, uint32_t nbPairs, bool pairState)
	{
		return sizeof(SnapshotHeader) + size_t(nb) * (sizeof(tgs::RigidBody) + 4 + 16 + 4) + size_t(ns) * (28 + 4 + 16) +
		       (pairState ? size_t(nbPairs) * (4 + sizeof(np::ManifoldRecord) + sizeof(tgs::FrictionState)) : 0);
	}
	int snapshot(uint32_t slot, std::vector<uint8_t>& out)
	{
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		const world::SceneDesc& d = hScenes[slot];
		const bool ps = params.persistent != 0;
		uint32_t nbPairs = 0, par = 0;
		if(ps)
		{
			GBPX_CUDA_TRY(cudaMemcpy(&nbPairs, pairCount.ptr + slot, 4, cudaMemcpyDeviceToHost));
			GBPX_CUDA_TRY(cudaMemcpy(&par, sceneParity.ptr + slot, 4, cudaMemcpyDeviceToHost));
			if(nbPairs > d.pairCap || par > 1u) return GBPX_ERR_STATE;
		}
		out.resize(snapshotBytes(d.nbBodies, d.nbStatics, nbPairs, ps));
		SnapshotHeader h = {SNAPSHOT_MAGIC, 1u, d.nbBodies, d.nbStatics, nbPairs, ps ? 1u : 0u, {0u, 0u}};
		uint8_t* o = out.data();
		memcpy(o, &h, sizeof(h));
		o += sizeof(h);
		auto get = [&](const void* src, size_t bytes) -> cudaError_t {
			const cudaError_t e = bytes ? cudaMemcpy(o, src, bytes, cudaMemcpyDeviceToHost) : cudaSuccess;
			o += bytes;
			return e;
		};
		const uint32_t b = d.bodyStart, st = d.staticStart, nb = d.nbBodies, ns = d.nbStatics;
		GBPX_CUDA_TRY(get(bodies.ptr + b, size_t(nb) * sizeof(tgs::RigidBody)));
		GBPX_CUDA_TRY(get(types.ptr + b, size_t(nb) * 4));
		GBPX_CUDA_TRY(get(geoms.ptr + b, size_t(nb) * 16));
		GBPX_CUDA_TRY(get(friction.ptr + b, size_t(nb) * 4));
		GBPX_CUDA_TRY(get(staticPose.ptr + 7 * size_t(st), size_t(ns) * 28));
		GBPX_CUDA_TRY(get(staticTypes.ptr + st, size_t(ns) * 4));
		GBPX_CUDA_TRY(get(staticGeoms.ptr + st, size_t(ns) * 16));
		if(ps)
		{
			GBPX_CUDA_TRY(get(pairs.ptr + d.pairStart, size_t(nbPairs) * 4));
			GBPX_CUDA_TRY(get(manifolds[par].ptr + d.pairStart, size_t(nbPairs) * sizeof(np::ManifoldRecord)));
			GBPX_CUDA_TRY(get(frictionState[par].ptr + d.pairStart, size_t(nbPairs) * sizeof(tgs::FrictionState)));
		}
		return GBPX_OK;
	}
	// The scene of a snapshot into slot `slot` (capacity checked by the caller).
	int restore(uint32_t slot, const uint8_t* in, size_t bytes)
	{
		SnapshotHeader h;
		if(bytes < sizeof(h)) return GBPX_ERR_INVALID;
		memcpy(&h, in, sizeof(h));
		const bool ps = h.pairState != 0;
		if(h.magic != SNAPSHOT_MAGIC || h.version != 1u || bytes != snapshotBytes(h.nbBodies, h.nbStatics, h.nbPairs, ps) ||
		   ps != (params.persistent != 0))
			return GBPX_ERR_INVALID;
		const world::SceneDesc& d = hScenes[slot];
		if(ps && h.nbPairs > d.pairCap) return GBPX_ERR_CAPACITY;
		const uint8_t* p = in + sizeof(h);
		const uint32_t nb = h.nbBodies, ns = h.nbStatics;
		const uint8_t* rigid = p;
		const int* ty = reinterpret_cast<const int*>(rigid + size_t(nb) * sizeof(tgs::RigidBody));
		const float* ge = reinterpret_cast<const float*>(reinterpret_cast<const uint8_t*>(ty) + size_t(nb) * 4);
		const float* fr = ge + size_t(nb) * 4;
		const float* sp7 = fr + nb;
		const int* sty = reinterpret_cast<const int*>(sp7 + size_t(ns) * 7);
		const float* sge = reinterpret_cast<const float*>(sty + ns);
		const uint8_t* pairState = reinterpret_cast<const uint8_t*>(sge + size_t(ns) * 4);
		int rc = admit(slot, nb, rigid, ty, ge, fr, ns, sp7, sty, sge);
		if(rc || !ps) return rc;
		// the pair list and its state into the buffer the slot reads next
		uint32_t par = 0;
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		GBPX_CUDA_TRY(cudaMemcpy(&par, sceneParity.ptr + slot, 4, cudaMemcpyDeviceToHost));
		if(par > 1u) return GBPX_ERR_STATE;
		const size_t pairsIn = h.nbPairs;
		GBPX_CUDA_TRY(cudaMemcpy(pairs.ptr + d.pairStart, pairState, pairsIn * 4, cudaMemcpyHostToDevice));
		GBPX_CUDA_TRY(cudaMemcpy(manifolds[par].ptr + d.pairStart, pairState + pairsIn * 4, pairsIn * sizeof(np::ManifoldRecord), cudaMemcpyHostToDevice));
		GBPX_CUDA_TRY(cudaMemcpy(frictionState[par].ptr + d.pairStart, pairState + pairsIn * (4 + sizeof(np::ManifoldRecord)),
		                         pairsIn * sizeof(tgs::FrictionState), cudaMemcpyHostToDevice));
		const uint32_t np32 = uint32_t(pairsIn);
		GBPX_CUDA_TRY(cudaMemcpy(pairCount.ptr + slot, &np32, 4, cudaMemcpyHostToDevice));
		return GBPX_OK;
	}

	void release()
	{
		if(stream) cudaStreamSynchronize(stream);
		if(graphExec) cudaGraphExecDestroy(graphExec);
		graphExec = nullptr;
		pairsPrev.release(); pairCountPrev.release(); prevSlot.release(); sceneParity.release();
		for(int k = 0; k < 2; k++) { manifolds[k].release(); frictionState[k].release(); }
		typeQueueSorted.release();
		scenes.release(); typeQueue.release(); slotScene.release(); activeCount.release(); recChunks.release(); nbConstraints.release(); nbPartitions.release(); prepQueue.release(); prepQueueSorted.release(); prepClass.release(); workOrder.release(); workCounter.release(); pairs.release(); pairCount.release(); contactCount.release();
		ordered.release(); consList.release(); tag.release(); progress.release(); maxNormal.release(); maxStatic.release();
		staticProgress.release(); partEnds.release(); status.release(); bodies.release(); types.release(); staticTypes.release();
		geoms.release(); staticGeoms.release(); contacts.release(); friction.release(); staticPose.release(); aabb.release();
		keys.release(); stats.release(); identity.release(); recs.release(); sceneAcc.release(); resList.release(); vel.release(); tx.release(); data.release(); pose.release(); hStage.release();
		if(sideStream) { cudaStreamSynchronize(sideStream); cudaStreamDestroy(sideStream); }
		sideStream = 0;
		for(int k = 0; k < 4; k++)
		{
			if(forkEv[k]) cudaEventDestroy(forkEv[k]);
			if(joinEv[k]) cudaEventDestroy(joinEv[k]);
			forkEv[k] = joinEv[k] = nullptr;
		}
		if(stream) cudaStreamDestroy(stream);
		stream = 0;
	}
};
} // namespace gbpx

using gbpx::World;

// Creates a world of nbScenes independent scenes.  Scene s owns
// sceneBodyCount[s] consecutive dynamic bodies (PxRigidBodyData records with
// shape type, 4 geometry floats and a friction coefficient each) and
// sceneStaticCount[s] consecutive static shapes (PxTransform pose, type,
// geometry; friction `staticFriction`).  params: dt, gravity xyz,
// contactDistance, toleranceLength, boundsMargin, bounceThreshold,
// frictionOffsetThreshold, correlationDistance, staticFriction (11 floats);
// iterations: nbPositionIterations, nbVelocityIterations.
GBPX_API int gbpx_world_create(uint32_t nbScenes, const uint32_t* sceneBodyCount, const uint32_t* sceneStaticCount, const void* rigidBodies,
                               const int* types, const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes,
                               const float* staticGeoms, const float* params, const uint32_t* iterations, uint32_t pairsPerBody,
                               void** outWorld)
{
	if(!outWorld || !nbScenes || !sceneBodyCount || !sceneStaticCount || !rigidBodies || !types || !geoms || !friction || !params ||
	   !iterations || !iterations[0] || !iterations[1] || !pairsPerBody)
		return GBPX_ERR_INVALID;
	gbpx::world::StepParams sp;
	sp.dt = params[0]; sp.gx = params[1]; sp.gy = params[2]; sp.gz = params[3];
	sp.contactDistance = params[4]; sp.toleranceLength = params[5]; sp.boundsMargin = params[6];
	sp.bounceThreshold = params[7]; sp.frictionOffsetThreshold = params[8]; sp.correlationDistance = params[9]; sp.staticFriction = params[10];
	sp.persistent = params[11] != 0.0f ? 1u : 0u;
	sp.nbPos = iterations[0]; sp.nbVel = iterations[1];
	sp.largeBodies = World::DEFAULT_LARGE_BODIES;
	sp.solveVariant = gbpx::world::RESIDENT_VARIANT;
	sp.resBytes = 0;       // set at creation
	sp.resStream = World::DEFAULT_RES_STREAM;
	if(!(sp.dt > 0.0f) || !(sp.contactDistance > 0.0f)) return GBPX_ERR_INVALID;
	for(uint32_t s = 0, b = 0; s < nbScenes; s++)
		for(uint32_t i = 0; i < sceneBodyCount[s]; i++, b++)
			if(uint32_t(types[b]) > 3u || types[b] == 1) return GBPX_ERR_INVALID;   // dynamic planes are not allowed
	World* w = new World;
	const int rc = w->create(nbScenes, sceneBodyCount, sceneStaticCount, rigidBodies, types, geoms, friction, staticPoses, staticTypes,
	                         staticGeoms, pairsPerBody, sp);
	if(rc) { w->release(); delete w; return rc; }
	*outWorld = w;
	return GBPX_OK;
}

GBPX_API void gbpx_world_release(void* w)
{
	if(!w) return;
	static_cast<World*>(w)->release();
	delete static_cast<World*>(w);
}

// Advances every scene by nbSteps on the device (asynchronous; state stays in
// HBM).  useGraph replays a captured CUDA graph of one step.
GBPX_API int gbpx_world_step(void* w, uint32_t nbSteps, int useGraph)
{
	gbpx::Zone zone("gbpx::world::step");
	if(!w) return GBPX_ERR_INVALID;
	return static_cast<World*>(w)->step(nbSteps, useGraph != 0);
}

GBPX_API int gbpx_world_synchronize(void* w)
{
	if(!w) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaStreamSynchronize(static_cast<World*>(w)->stream));
	return GBPX_OK;
}

// Copies every dynamic body (PxRigidBodyData) to / from host memory.
GBPX_API int gbpx_world_get_bodies(void* wv, void* outRigid)
{
	World* w = static_cast<World*>(wv);
	if(!w || !outRigid) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRigid, w->bodies.ptr, size_t(w->nbBodies) * sizeof(gbpx::tgs::RigidBody), cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

GBPX_API int gbpx_world_set_bodies(void* wv, const void* rigid)
{
	World* w = static_cast<World*>(wv);
	if(!w || !rigid) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(w->bodies.ptr, rigid, size_t(w->nbBodies) * sizeof(gbpx::tgs::RigidBody), cudaMemcpyHostToDevice, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

// Per-scene status words (bit 0: pair buffer overflow, bit 1: partition
// overflow), cleared after reading.
GBPX_API int gbpx_world_status(void* wv, uint32_t* outStatus)
{
	World* w = static_cast<World*>(wv);
	if(!w || !outStatus) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(outStatus, w->status.ptr, size_t(w->nbScenes) * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaMemsetAsync(w->status.ptr, 0, size_t(w->nbScenes) * 4, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

// nbScenes, nbBodies, nbStatics, pair slots, persistent grid blocks of the
// broadphase, device bytes, kernels launched per step, reserved (0)
GBPX_API int gbpx_world_info(void* wv, uint64_t* out8)
{
	World* w = static_cast<World*>(wv);
	if(!w || !out8) return GBPX_ERR_INVALID;
	out8[0] = w->nbScenes; out8[1] = w->nbBodies; out8[2] = w->nbStatics; out8[3] = w->nbPairSlots; out8[4] = w->gridBlocks;
	out8[5] = w->deviceBytes;
	out8[6] = World::KERNELS_PER_STEP + 1u + (w->launchLarge() ? (w->resident() ? 2u : 3u) : 0u) + (w->params.persistent ? 1u : 0u);
	out8[7] = w->params.largeBodies;
	return GBPX_OK;
}

// Pair list of one scene after the last step: (id0 << 16 | id1) keys sorted,
// statics numbered after the scene's dynamic bodies; and contact counts.
GBPX_API int gbpx_world_scene_pairs(void* wv, uint32_t scene, uint32_t* outKeys, uint32_t* outContactCounts, uint32_t capacity,
                                    uint32_t* outCount)
{
	World* w = static_cast<World*>(wv);
	if(!w || scene >= w->nbScenes || !outCount) return GBPX_ERR_INVALID;
	uint32_t count = 0;
	GBPX_CUDA_TRY(cudaMemcpyAsync(&count, w->pairCount.ptr + scene, 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	*outCount = count;
	const uint32_t m = count < capacity ? count : capacity;
	const uint32_t start = w->hScenes[scene].pairStart;
	if(m && outKeys) GBPX_CUDA_TRY(cudaMemcpyAsync(outKeys, w->pairs.ptr + start, size_t(m) * 4, cudaMemcpyDeviceToHost, w->stream));
	if(m && outContactCounts)
		GBPX_CUDA_TRY(cudaMemcpyAsync(outContactCounts, w->contactCount.ptr + start, size_t(m) * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

// Times nbSteps steps with CUDA events on the world's stream (device-resident
// state, no host traffic); returns milliseconds.
GBPX_API int gbpx_world_time_steps(void* wv, uint32_t nbSteps, int useGraph, float* outMs)
{
	World* w = static_cast<World*>(wv);
	if(!w || !outMs) return GBPX_ERR_INVALID;
	if(useGraph && (!w->graphExec || w->graphSteps != 1))
	{
		const int rc = w->capture(1);
		if(rc) return rc;
	}
	cudaEvent_t e0, e1;
	GBPX_CUDA_TRY(cudaEventCreate(&e0));
	GBPX_CUDA_TRY(cudaEventCreate(&e1));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	GBPX_CUDA_TRY(cudaEventRecord(e0, w->stream));
	const int rc = w->step(nbSteps, useGraph != 0);
	GBPX_CUDA_TRY(cudaEventRecord(e1, w->stream));
	GBPX_CUDA_TRY(cudaEventSynchronize(e1));
	GBPX_CUDA_TRY(cudaEventElapsedTime(outMs, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

// Steps scenes [first, first + count) one scene per launch (no cross-scene
// batching, no graph) and returns the elapsed milliseconds (CUDA events).
GBPX_API int gbpx_world_time_plain(void* wv, uint32_t first, uint32_t count, float* outMs)
{
	World* w = static_cast<World*>(wv);
	if(!w || !outMs) return GBPX_ERR_INVALID;
	cudaEvent_t e0, e1;
	GBPX_CUDA_TRY(cudaEventCreate(&e0));
	GBPX_CUDA_TRY(cudaEventCreate(&e1));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	GBPX_CUDA_TRY(cudaEventRecord(e0, w->stream));
	const int rc = w->stepPlain(first, count);
	GBPX_CUDA_TRY(cudaEventRecord(e1, w->stream));
	GBPX_CUDA_TRY(cudaEventSynchronize(e1));
	GBPX_CUDA_TRY(cudaEventElapsedTime(outMs, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

// Totals of the last step: pairs, pairs with contacts (constraints), contacts,
// bytes of packed constraint rows.
GBPX_API int gbpx_world_stats(void* wv, uint64_t* out4)
{
	World* w = static_cast<World*>(wv);
	if(!w || !out4) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemsetAsync(w->stats.ptr, 0, 4 * 8, w->stream));
	gbpx::world::statsKernel<<<w->nbScenes, 256, 0, w->stream>>>(w->scenes.ptr, w->nbScenes, w->pairCount.ptr, w->contactCount.ptr,
	                                                              w->nbConstraints.ptr, w->nbPartitions.ptr, w->recChunks.ptr, w->stats.ptr);
	GBPX_CUDA_TRY(cudaGetLastError());
	GBPX_CUDA_TRY(cudaMemcpyAsync(out4, w->stats.ptr, 4 * 8, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

// Per scene after the last step: constraints, partitions, bytes of packed
// constraint rows, and the widest partition (constraints) -- the figures that
// set the solve's on-chip footprint and critical path.  out4: 4 words per scene.
GBPX_API int gbpx_world_solve_profile(void* wv, uint32_t* out4)
{
	World* w = static_cast<World*>(wv);
	if(!w || !out4) return GBPX_ERR_INVALID;
	const uint32_t S = w->nbScenes;
	std::vector<uint32_t> nc(S), np(S), ends(size_t(S) * gbpx::world::MAX_PARTITIONS);
	std::vector<uint8_t> chunks(w->nbPairSlots);
	GBPX_CUDA_TRY(cudaMemcpyAsync(nc.data(), w->nbConstraints.ptr, S * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaMemcpyAsync(np.data(), w->nbPartitions.ptr, S * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaMemcpyAsync(ends.data(), w->partEnds.ptr, ends.size() * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaMemcpyAsync(chunks.data(), w->recChunks.ptr, chunks.size(), cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	for(uint32_t s = 0; s < S; s++)
	{
		const uint32_t p = np[s], n = p ? nc[s] : 0;
		uint64_t bytes = 0;
		for(uint32_t r = 0; r < n; r++) bytes += 16u * chunks[w->hScenes[s].pairStart + r];
		uint32_t widest = 0, begin = 0;
		for(uint32_t k = 0; k < p; k++)
		{
			const uint32_t e = ends[size_t(s) * gbpx::world::MAX_PARTITIONS + k];
			widest = std::max(widest, e - begin);
			begin = e;
		}
		out4[4 * s + 0] = n; out4[4 * s + 1] = p; out4[4 * s + 2] = uint32_t(bytes); out4[4 * s + 3] = widest;
	}
	return GBPX_OK;
}

// Scenes of more than `largeBodies` solver bodies (bodies + statics) run their
// broadphase, batching and solve one block of 8 warps per scene; smaller ones
// one warp per scene (default 512).  The arithmetic is the same either way.
GBPX_API int gbpx_world_set_large_bodies(void* wv, uint32_t largeBodies)
{
	World* w = static_cast<World*>(wv);
	if(!w) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	w->params.largeBodies = largeBodies;
	if(w->graphExec)
	{
		cudaGraphExecDestroy(w->graphExec);
		w->graphExec = nullptr;
	}
	return GBPX_OK;
}

GBPX_API int gbpx_world_set_solve_variant(void* wv, uint32_t variant);

// Persistent blocks per SM of the row preparation and of the capsule-box and
// box-box narrowphase kernels (0: as many as fit, the default).  Their threads
// keep large working sets in local memory; fewer in flight keeps it on chip.
// Results do not depend on it.
GBPX_API int gbpx_world_set_occupancy(void* wv, uint32_t prepBlocksPerSm, uint32_t narrowphaseBlocksPerSm)
{
	World* w = static_cast<World*>(wv);
	if(!w) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	w->prepPerSm = prepBlocksPerSm;
	w->npHeavyPerSm = narrowphaseBlocksPerSm;
	if(w->graphExec)
	{
		cudaGraphExecDestroy(w->graphExec);
		w->graphExec = nullptr;
	}
	return GBPX_OK;
}

// ---- Autotuner of the block-per-scene threshold and the solve staging slot ----
// The scene stages run warp-per-scene or block-per-scene kernels by scene size
// (gbpx_world_set_large_bodies).  The best threshold depends on the scene-size
// histogram: the autotuner takes a size-stratified sample of the world's scenes
// in their current state into a temporary world, times a few graph-replayed
// steps per candidate threshold there, and sets the fastest on the world.  The
// choice is cached per histogram (scene counts per power-of-two size bucket,
// quantised to 1/32 of the scenes), so worlds of the same size mix reuse it.
namespace
{
std::string histogramKey(const std::vector<gbpx::world::SceneDesc>& sc)
{
	uint32_t buckets[32] = {};
	for(const auto& d : sc)
	{
		uint32_t b = 0;
		while((1u << b) < d.nbBodies + d.nbStatics) b++;
		buckets[b]++;
	}
	std::string key;
	for(uint32_t b = 0; b < 32; b++)
	{
		const uint32_t q = uint32_t((uint64_t(buckets[b]) * 32 + sc.size() / 2) / sc.size());
		key += std::to_string(q) + ",";
	}
	return key;
}
// a tuned configuration: block-per-scene threshold, solve kernel, and the
// blocks per SM of the preparation and heavy narrowphase kernels (0 = as many
// as fit)
struct Tuning
{
	uint32_t largeBodies, solveVariant, prepPerSm, npHeavyPerSm, resStream;
};
std::map<std::string, Tuning>& tunedConfigs()
{
	static std::map<std::string, Tuning> m;
	return m;
}
} // namespace

GBPX_API int gbpx_world_set_resident_stream(void* wv, uint32_t levels);
GBPX_API int gbpx_world_autotune(void* wv, uint32_t sampleScenes, uint32_t steps, uint32_t* outLargeBodies, uint32_t* outSolveVariant,
                                 float* outMs)
{
	World* w = static_cast<World*>(wv);
	if(!w || !sampleScenes || !steps || !outLargeBodies || !outSolveVariant) return GBPX_ERR_INVALID;
	const std::string key = histogramKey(w->hScenes);
	auto& cache = tunedConfigs();
	auto hit = cache.find(key);
	if(hit != cache.end())
	{
		const Tuning& c = hit->second;
		*outLargeBodies = c.largeBodies;
		*outSolveVariant = c.solveVariant;
		if(outMs) *outMs = 0.0f;
		int rc = gbpx_world_set_large_bodies(wv, c.largeBodies);
		rc = rc ? rc : gbpx_world_set_solve_variant(wv, c.solveVariant);
		rc = rc ? rc : gbpx_world_set_resident_stream(wv, c.resStream);
		return rc ? rc : gbpx_world_set_occupancy(wv, c.prepPerSm, c.npHeavyPerSm);
	}
	// size-stratified sample: every k-th scene in order of size
	std::vector<uint32_t> order(w->nbScenes);
	std::iota(order.begin(), order.end(), 0u);
	std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return w->hScenes[x].nbBodies < w->hScenes[y].nbBodies; });
	const uint32_t m = std::min(sampleScenes, w->nbScenes);
	std::vector<uint32_t> pick(m);
	for(uint32_t k = 0; k < m; k++) pick[k] = order[uint32_t((uint64_t(k) * w->nbScenes + w->nbScenes / 2) / m) % w->nbScenes];
	// the sample's arrays, read back from the world (current body state)
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	std::vector<uint32_t> bc(m), sc(m);
	std::vector<gbpx::tgs::RigidBody> rb;
	std::vector<int> ty, sty;
	std::vector<float4> ge, sge;
	std::vector<float> fr, sp7;
	for(uint32_t k = 0; k < m; k++)
	{
		const gbpx::world::SceneDesc& d = w->hScenes[pick[k]];
		bc[k] = d.nbBodies;
		sc[k] = d.nbStatics;
		const size_t b0 = rb.size(), s0 = sty.size();
		rb.resize(b0 + d.nbBodies); ty.resize(b0 + d.nbBodies); ge.resize(b0 + d.nbBodies); fr.resize(b0 + d.nbBodies);
		sty.resize(s0 + d.nbStatics); sge.resize(s0 + d.nbStatics); sp7.resize(7 * (s0 + d.nbStatics));
		GBPX_CUDA_TRY(cudaMemcpy(rb.data() + b0, w->bodies.ptr + d.bodyStart, size_t(d.nbBodies) * sizeof(gbpx::tgs::RigidBody), cudaMemcpyDeviceToHost));
		GBPX_CUDA_TRY(cudaMemcpy(ty.data() + b0, w->types.ptr + d.bodyStart, size_t(d.nbBodies) * 4, cudaMemcpyDeviceToHost));
		GBPX_CUDA_TRY(cudaMemcpy(ge.data() + b0, w->geoms.ptr + d.bodyStart, size_t(d.nbBodies) * 16, cudaMemcpyDeviceToHost));
		GBPX_CUDA_TRY(cudaMemcpy(fr.data() + b0, w->friction.ptr + d.bodyStart, size_t(d.nbBodies) * 4, cudaMemcpyDeviceToHost));
		if(d.nbStatics)
		{
			GBPX_CUDA_TRY(cudaMemcpy(sty.data() + s0, w->staticTypes.ptr + d.staticStart, size_t(d.nbStatics) * 4, cudaMemcpyDeviceToHost));
			GBPX_CUDA_TRY(cudaMemcpy(sge.data() + s0, w->staticGeoms.ptr + d.staticStart, size_t(d.nbStatics) * 16, cudaMemcpyDeviceToHost));
			GBPX_CUDA_TRY(cudaMemcpy(sp7.data() + 7 * s0, w->staticPose.ptr + 7 * size_t(d.staticStart), size_t(d.nbStatics) * 28, cudaMemcpyDeviceToHost));
		}
	}
	World* t = new World;
	int rc = t->create(m, bc.data(), sc.data(), rb.data(), ty.data(), reinterpret_cast<const float*>(ge.data()), fr.data(),
	                   sp7.empty() ? nullptr : sp7.data(), sty.empty() ? nullptr : sty.data(),
	                   sge.empty() ? nullptr : reinterpret_cast<const float*>(sge.data()), w->pairsPerBody, w->params);
	if(rc) { t->release(); delete t; return rc; }
	t->params.resStream = World::DEFAULT_RES_STREAM;
	// the copy starts without pair state (manifolds, friction patches): a few
	// steps fill it, so that every candidate is timed in the steady state
	rc = t->step(6, true);
	if(rc) { t->release(); delete t; return rc; }
	// candidates that classify the sample differently
	const uint32_t cands[] = {64u, 128u, 256u, 512u, 1024u, 2048u, 0xffffffffu};
	std::vector<uint32_t> sizes;
	for(uint32_t k = 0; k < m; k++) sizes.push_back(bc[k] + sc[k]);
	cudaEvent_t e0, e1;
	GBPX_CUDA_TRY(cudaEventCreate(&e0));
	GBPX_CUDA_TRY(cudaEventCreate(&e1));
	auto timeConfig = [&](uint32_t threshold, uint32_t variant, float& ms) -> int {
		t->params.largeBodies = threshold;
		t->params.solveVariant = variant;
		if(t->graphExec) { cudaGraphExecDestroy(t->graphExec); t->graphExec = nullptr; }
		int r = t->step(2, true);
		if(r) return r;
		GBPX_CUDA_TRY(cudaEventRecord(e0, t->stream));
		r = t->step(steps, true);
		if(r) return r;
		GBPX_CUDA_TRY(cudaEventRecord(e1, t->stream));
		GBPX_CUDA_TRY(cudaEventSynchronize(e1));
		GBPX_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
		return GBPX_OK;
	};
	// a later candidate replaces the incumbent (the defaults first) only when it is
	// at least 2 % faster: the copy's timing of a few steps varies by about 1 %, and
	// its state differs a little from the world's own
	const float TUNE_MARGIN = 0.98f;
	// the threshold first (default staging), then the staging slot at that threshold
	uint32_t best = w->params.largeBodies, bestVariant = w->params.solveVariant;
	float bestMs = 3.4e38f;
	int lastLarge = -1;
	for(uint32_t c : cands)
	{
		const int nLarge = int(std::count_if(sizes.begin(), sizes.end(), [&](uint32_t x) { return x > c; }));
		if(nLarge == lastLarge) continue;
		lastLarge = nLarge;
		float ms = 0.0f;
		rc = timeConfig(c, bestVariant, ms);
		if(rc) break;
		if(ms < bestMs) { bestMs = ms; best = c; }
	}
	const bool anySmall = std::any_of(sizes.begin(), sizes.end(), [&](uint32_t x) { return x <= best; });
	for(uint32_t v = 0; v <= gbpx::world::RESIDENT_VARIANT && !rc; v++)
	{
		// the staging variants only change the solve of scenes below the threshold
		if(v == bestVariant || (v != gbpx::world::RESIDENT_VARIANT && !anySmall)) continue;
		float ms = 0.0f;
		rc = timeConfig(best, v, ms);
		if(!rc && ms < bestMs * TUNE_MARGIN) { bestMs = ms; bestVariant = v; }
	}
	// the resident solve's streamed-row levels
	uint32_t bestStream = World::DEFAULT_RES_STREAM;
	if(bestVariant == gbpx::world::RESIDENT_VARIANT)
		for(uint32_t d = 0; d <= 2 && !rc; d++)
		{
			if(d == World::DEFAULT_RES_STREAM) continue;
			t->params.resStream = d;
			float ms = 0.0f;
			rc = timeConfig(best, bestVariant, ms);
			if(!rc && ms < bestMs * TUNE_MARGIN) { bestMs = ms; bestStream = d; }
		}
	t->params.resStream = bestStream;
	// then the blocks per SM of the row preparation (rows per CTA wave) and of the
	// two heavy narrowphase kinds (pairs per CTA wave), one after the other
	uint32_t bestPrep = t->prepPerSm, bestNp = t->npHeavyPerSm;
	for(uint32_t c : {2u, 3u, 4u})
	{
		if(rc) break;
		t->prepPerSm = c;
		float ms = 0.0f;
		rc = timeConfig(best, bestVariant, ms);
		if(!rc && ms < bestMs * TUNE_MARGIN) { bestMs = ms; bestPrep = c; }
	}
	t->prepPerSm = bestPrep;
	for(uint32_t c : {1u, 2u, 3u})
	{
		if(rc) break;
		t->npHeavyPerSm = c;
		float ms = 0.0f;
		rc = timeConfig(best, bestVariant, ms);
		if(!rc && ms < bestMs * TUNE_MARGIN) { bestMs = ms; bestNp = c; }
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	t->release();
	delete t;
	if(rc) return rc;
	cache[key] = Tuning{best, bestVariant, bestPrep, bestNp, bestStream};
	*outLargeBodies = best;
	*outSolveVariant = bestVariant;
	if(outMs) *outMs = bestMs / float(steps);
	rc = gbpx_world_set_large_bodies(wv, best);
	rc = rc ? rc : gbpx_world_set_solve_variant(wv, bestVariant);
	rc = rc ? rc : gbpx_world_set_resident_stream(wv, bestStream);
	return rc ? rc : gbpx_world_set_occupancy(wv, bestPrep, bestNp);
}

// The world's current tuning: out4 = block-per-scene threshold, solve kernel,
// preparation blocks per SM, heavy narrowphase blocks per SM (0 = as many as fit).
GBPX_API int gbpx_world_tuning(void* wv, uint32_t* out5)
{
	World* w = static_cast<World*>(wv);
	if(!w || !out5) return GBPX_ERR_INVALID;
	out5[0] = w->params.largeBodies;
	out5[1] = w->params.solveVariant;
	out5[2] = w->prepPerSm;
	out5[3] = w->npHeavyPerSm;
	out5[4] = w->params.resStream;
	return GBPX_OK;
}

// Streamed rows in the resident solve (0 .. 3, default 1): a scene whose rows
// and velocities need a level above `levels` is solved one level deeper (by a
// group of at least two warps) with its rows streamed chunk by chunk through a
// two-slot ring in its slice, so more scenes are in flight per SM; scenes too
// large for any slice stream their rows too (levels > 0).  Results do not
// depend on it.
GBPX_API int gbpx_world_set_resident_stream(void* wv, uint32_t levels)
{
	World* w = static_cast<World*>(wv);
	if(!w || levels + 1 >= gbpx::world::RES_LEVELS) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	w->params.resStream = levels;
	if(w->graphExec)
	{
		cudaGraphExecDestroy(w->graphExec);
		w->graphExec = nullptr;
	}
	return GBPX_OK;
}

// Solve kernel of the world.  8 (the default): the resident solve, every
// scene's rows and velocities on chip for all iterations.  0-7: the
// warp-per-scene solve, whose variants 0-2 keep the body velocities in shared
// memory and stage rows in 0 / 256 / 512 bytes per lane, 3-5 the same with the
// velocities left in HBM, 6 / 7 stage 400 bytes per lane with the velocities on
// chip / in HBM (a smaller workspace leaves room for more warps per SM).
// Results do not depend on it.
GBPX_API int gbpx_world_set_solve_variant(void* wv, uint32_t variant)
{
	World* w = static_cast<World*>(wv);
	if(!w || variant > gbpx::world::RESIDENT_VARIANT) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	w->params.solveVariant = variant;
	if(w->graphExec)
	{
		cudaGraphExecDestroy(w->graphExec);
		w->graphExec = nullptr;
	}
	return GBPX_OK;
}

// Pairs of each pair kind in the last step (sphere-sphere, sphere-plane,
// sphere-capsule, sphere-box, plane-capsule, plane-box, capsule-capsule,
// capsule-box, box-box): 9 counts.
GBPX_API int gbpx_world_kind_counts(void* wv, uint32_t* out9)
{
	World* w = static_cast<World*>(wv);
	if(!w || !out9) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(out9, w->workCounter.ptr + 8, 9 * 4, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(w->stream));
	return GBPX_OK;
}

// Average device time of each kernel of a step over nbSteps un-captured steps
// (CUDA events between the launches on the world's stream), in launch order:
// broadphase, the narrowphase kernels per pair kind, batching, row
// preparation, solve.  outMs has KERNELS_PER_STEP entries (gbpx_world_info).
GBPX_API int gbpx_world_time_stages(void* wv, uint32_t nbSteps, float* outMs)
{
	World* w = static_cast<World*>(wv);
	if(!w || !outMs || !nbSteps) return GBPX_ERR_INVALID;
	return w->timeStages(nbSteps, outMs);
}

// End-to-end step through host memory: uploads the bodies from `rigidIn`
// (host, PxRigidBodyData), advances every scene by nbSteps and downloads them
// into `rigidOut`; returns the elapsed milliseconds measured with CUDA events
// around the copies and the step.
GBPX_API int gbpx_world_step_host(void* wv, const void* rigidIn, void* rigidOut, uint32_t nbSteps, int useGraph, float* outMs)
{
	gbpx::Zone zone("gbpx::world::stepHost");
	World* w = static_cast<World*>(wv);
	if(!w || !rigidIn || !rigidOut) return GBPX_ERR_INVALID;
	if(useGraph && (!w->graphExec || w->graphSteps != 1))
	{
		const int rc = w->capture(1);
		if(rc) return rc;
	}
	cudaEvent_t e0, e1;
	GBPX_CUDA_TRY(cudaEventCreate(&e0));
	GBPX_CUDA_TRY(cudaEventCreate(&e1));
	GBPX_CUDA_TRY(cudaEventRecord(e0, w->stream));
	const size_t bytes = size_t(w->nbBodies) * sizeof(gbpx::tgs::RigidBody);
	GBPX_CUDA_TRY(cudaMemcpyAsync(w->bodies.ptr, rigidIn, bytes, cudaMemcpyHostToDevice, w->stream));
	const int rc = w->step(nbSteps, useGraph != 0);
	GBPX_CUDA_TRY(cudaMemcpyAsync(rigidOut, w->bodies.ptr, bytes, cudaMemcpyDeviceToHost, w->stream));
	GBPX_CUDA_TRY(cudaEventRecord(e1, w->stream));
	GBPX_CUDA_TRY(cudaEventSynchronize(e1));
	if(outMs) GBPX_CUDA_TRY(cudaEventElapsedTime(outMs, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

// Pinned host allocation for world body arrays (fast copies); free with gbpx_host_free.
GBPX_API int gbpx_host_alloc(size_t bytes, void** out)
{
	if(!out) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMallocHost(out, bytes));
	return GBPX_OK;
}

GBPX_API void gbpx_host_free(void* p)
{
	if(p) cudaFreeHost(p);
}

// ------------------------------------------------------------------ serving
// A request loop over a live pool of scenes kept resident in HBM.  Scenes are
// admitted into fixed-capacity slots grouped by body-count class; each class
// is a lane (a world of slots with its own stream and captured step), so
// small scenes never wait behind large ones.  A request "advance scene k by n
// steps" queues behind the scene's earlier requests; every pump issues one
// step per lane over the scenes that still owe steps (continuous batching:
// requests that arrive while a step runs join the next one), with up to two
// steps in flight per lane.  A scene's arithmetic does not depend on which
// other scenes share its step.
namespace gbpx
{
struct Server
{
	struct Request { uint64_t tag; uint64_t target; double arrival; };
	struct Scene { uint32_t lane = 0, slot = 0, nbBodies = 0; bool live = false; uint64_t requested = 0, issued = 0, done = 0; std::deque<Request> reqs; };
	struct Lane
	{
		World w;
		uint32_t capacity = 0, staticCap = 0, base = 0, slots = 0;
		std::vector<uint32_t> freeSlots;
		uint32_t* pinned[2] = {nullptr, nullptr};   // active list + count per in-flight step
		cudaEvent_t ev[2] = {nullptr, nullptr};
		std::vector<uint32_t> inflight[2];
		int head = 0, nbInflight = 0;
	};
	std::vector<Lane*> lanes;
	std::vector<Scene> scenes;
	std::vector<uint64_t> doneTags;
	std::vector<double> doneLatency;
	uint64_t bodySteps = 0, steps = 0;
	std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

	double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

	// Device bytes of one slot of `capacity` bodies and `statics` statics (the world layout).
	static size_t slotBytes(uint32_t capacity, uint32_t statics, uint32_t pairsPerBody, bool persistent)
	{
		const size_t pair = World::pow2(capacity * pairsPerBody + capacity * statics);
		const size_t key = World::pow2(capacity);
		const size_t persistentPair = persistent ? 16 + 2 * (sizeof(np::ManifoldRecord) + sizeof(tgs::FrictionState)) : 0;
		return pair * (4 + 128 + 4 * 4 + 4 + 4 * world::NB_KINDS + 4 + 4 + sizeof(tgs::ConstraintRecord) + persistentPair) +
		       size_t(capacity) * (96 + 4 + 16 + 4 + 24) +
		       size_t(capacity + statics) * (sizeof(tgs::BodyVel) + sizeof(tgs::BodyTx) + sizeof(tgs::BodyData) + sizeof(Tr) + 16) + key * 8 +
		       statics * 48 + world::MAX_PARTITIONS * 4 + 64;
	}

	int create(uint32_t nbClasses, const uint32_t* capacity, const uint32_t* slots, uint32_t staticsPerSlot, uint32_t pairsPerBody,
	           const world::StepParams& sp, uint32_t lanesPerClass)
	{
		uint32_t base = 0;
		for(uint32_t c = 0; c < nbClasses; c++)
		{
			// a class's slots split over lanesPerClass lanes: each lane steps its own
			// scenes on its own stream, so a step covers fewer scenes and lanes overlap
			const uint32_t k = std::max(1u, std::min(lanesPerClass, slots[c]));
			for(uint32_t j = 0; j < k; j++)
			{
				const uint32_t laneSlots = slots[c] / k + (j < slots[c] % k ? 1u : 0u);
				if(!laneSlots) continue;
				Lane* L = new Lane;
				lanes.push_back(L);
				L->capacity = capacity[c];
				L->slots = laneSlots;
				L->staticCap = staticsPerSlot;
				L->base = base;
				std::vector<uint32_t> cap(laneSlots, capacity[c]), st(laneSlots, staticsPerSlot);
				int rc = L->w.create(laneSlots, cap.data(), st.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, pairsPerBody, sp);
				if(rc) return rc;
				rc = L->w.capture(1);
				if(rc) return rc;
				for(uint32_t q = laneSlots; q > 0; q--) L->freeSlots.push_back(q - 1);
				for(int i = 0; i < 2; i++)
				{
					GBPX_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&L->pinned[i]), (size_t(laneSlots) + 1) * 4, cudaHostAllocDefault));
					GBPX_CUDA_TRY(cudaEventCreateWithFlags(&L->ev[i], cudaEventDisableTiming));
				}
				base += laneSlots;
			}
		}
		scenes.resize(base);
		return lanes.empty() ? GBPX_ERR_INVALID : GBPX_OK;
	}

	int admit(uint32_t nb, const void* rigid, const int* types, const float* geoms, const float* friction, uint32_t ns, const float* staticPoses,
	          const int* staticTypes, const float* staticGeoms, uint32_t* outScene)
	{
		// the smallest class that holds the scene; among its lanes, the one with the most free slots
		Lane* best = nullptr;
		for(Lane* L : lanes)
			if(L->capacity >= nb && !L->freeSlots.empty() && ns <= L->staticCap &&
			   (!best || L->capacity < best->capacity || (L->capacity == best->capacity && L->freeSlots.size() > best->freeSlots.size())))
				best = L;
		if(!best) return GBPX_ERR_BUDGET;
		const uint32_t slot = best->freeSlots.back();
		const int rc = best->w.admit(slot, nb, rigid, types, geoms, friction, ns, staticPoses, staticTypes, staticGeoms);
		if(rc) return rc;
		best->freeSlots.pop_back();
		const uint32_t id = best->base + slot;
		Scene& s = scenes[id];
		s = Scene();
		s.lane = uint32_t(std::find(lanes.begin(), lanes.end(), best) - lanes.begin());
		s.slot = slot;
		s.nbBodies = nb;
		s.live = true;
		*outScene = id;
		return GBPX_OK;
	}

	// Snapshot of a scene that owes no steps (World::snapshot's layout);
	// *outBytes is its size, and out (capacity bytes) receives it unless null.
	int snapshotScene(uint32_t id, void* out, uint64_t capacity, uint64_t* outBytes)
	{
		if(id >= scenes.size() || !scenes[id].live || !outBytes) return GBPX_ERR_INVALID;
		const Scene& s = scenes[id];
		if(s.done != s.requested) return GBPX_ERR_STATE;   // owes steps
		std::vector<uint8_t> blob;
		const int rc = lanes[s.lane]->w.snapshot(s.slot, blob);
		if(rc) return rc;
		*outBytes = blob.size();
		if(!out) return GBPX_OK;
		if(capacity < blob.size()) return GBPX_ERR_CAPACITY;
		memcpy(out, blob.data(), blob.size());
		return GBPX_OK;
	}

	// A snapshot admitted as a new scene (the smallest class that holds its
	// bodies, statics and pairs), continuing where the snapshot was taken.
	int restoreScene(const void* snap, uint64_t bytes, uint32_t* outScene)
	{
		World::SnapshotHeader h;
		if(!snap || !outScene || bytes < sizeof(h)) return GBPX_ERR_INVALID;
		memcpy(&h, snap, sizeof(h));
		Lane* best = nullptr;
		for(Lane* L : lanes)
		{
			const uint32_t pairCap = L->w.hScenes.empty() ? 0u : L->w.hScenes[0].pairCap;   // every slot of a lane alike
			if(L->capacity >= h.nbBodies && !L->freeSlots.empty() && h.nbStatics <= L->staticCap && h.nbPairs <= pairCap &&
			   (!best || L->capacity < best->capacity || (L->capacity == best->capacity && L->freeSlots.size() > best->freeSlots.size())))
				best = L;
		}
		if(!best) return GBPX_ERR_BUDGET;
		const uint32_t slot = best->freeSlots.back();
		const int rc = best->w.restore(slot, static_cast<const uint8_t*>(snap), bytes);
		if(rc) return rc;
		best->freeSlots.pop_back();
		const uint32_t id = best->base + slot;
		Scene& s = scenes[id];
		s = Scene();
		s.lane = uint32_t(std::find(lanes.begin(), lanes.end(), best) - lanes.begin());
		s.slot = slot;
		s.nbBodies = h.nbBodies;
		s.live = true;
		*outScene = id;
		return GBPX_OK;
	}

	int retire(uint32_t id)
	{
		if(id >= scenes.size() || !scenes[id].live) return GBPX_ERR_INVALID;
		Scene& s = scenes[id];
		if(s.done != s.requested) return GBPX_ERR_STATE;   // owes steps
		s.live = false;
		lanes[s.lane]->freeSlots.push_back(s.slot);
		return GBPX_OK;
	}

	int submit(uint32_t id, uint32_t nbSteps, uint64_t tag, double arrival)
	{
		if(id >= scenes.size() || !scenes[id].live || !nbSteps) return GBPX_ERR_INVALID;
		Scene& s = scenes[id];
		s.requested += nbSteps;
		s.reqs.push_back(Request{tag, s.requested, arrival < 0.0 ? now() : arrival});
		return GBPX_OK;
	}

	// Completes finished steps and issues new ones; returns the number of steps issued.
	int pump(uint32_t* outIssued)
	{
		uint32_t issued = 0;
		for(Lane* L : lanes)
		{
			while(L->nbInflight)
			{
				const int tail = (L->head + 2 - L->nbInflight) & 1;
				const cudaError_t q = cudaEventQuery(L->ev[tail]);
				if(q == cudaErrorNotReady) break;
				if(q != cudaSuccess) return GBPX_ERR_CUDA;
				const double t = now();
				for(uint32_t slot : L->inflight[tail])
				{
					Scene& s = scenes[L->base + slot];
					s.done++;
					bodySteps += s.nbBodies;
					while(!s.reqs.empty() && s.reqs.front().target <= s.done)
					{
						doneTags.push_back(s.reqs.front().tag);
						doneLatency.push_back(t - s.reqs.front().arrival);
						s.reqs.pop_front();
					}
				}
				steps++;
				L->nbInflight--;
			}
			if(L->nbInflight == 2) continue;
			std::vector<uint32_t>& list = L->inflight[L->head];
			list.clear();
			for(uint32_t slot = 0; slot < L->slots; slot++)
			{
				const Scene& s = scenes[L->base + slot];
				if(s.live && s.issued < s.requested) list.push_back(slot);
			}
			if(list.empty()) continue;
			std::stable_sort(list.begin(), list.end(),
			                 [&](uint32_t x, uint32_t y) { return scenes[L->base + x].nbBodies > scenes[L->base + y].nbBodies; });
			uint32_t* buf = L->pinned[L->head];
			std::copy(list.begin(), list.end(), buf);
			buf[L->slots] = uint32_t(list.size());
			GBPX_CUDA_TRY(cudaMemcpyAsync(L->w.workOrder.ptr, buf, list.size() * 4, cudaMemcpyHostToDevice, L->w.stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(L->w.activeCount.ptr, buf + L->slots, 4, cudaMemcpyHostToDevice, L->w.stream));
			GBPX_CUDA_TRY(cudaGraphLaunch(L->w.graphExec, L->w.stream));
			GBPX_CUDA_TRY(cudaEventRecord(L->ev[L->head], L->w.stream));
			for(uint32_t slot : list) scenes[L->base + slot].issued++;
			L->head ^= 1;
			L->nbInflight++;
			issued++;
		}
		if(outIssued) *outIssued = issued;
		return GBPX_OK;
	}

	// Library of scenes the load admits (one static shape each): bodies and
	// shapes of scene k at offsets[k] .. offsets[k + 1].
	struct Library
	{
		uint32_t count;
		const uint32_t* offsets;
		const tgs::RigidBody* rigid;
		const int* types;
		const float* geoms;
		const float* friction;
		const float* staticPoses;   // 7 floats per scene
		const int* staticTypes;
		const float* staticGeoms;   // 4 floats per scene
	};

	// The open-loop serving load, run natively: Poisson arrivals at `rate` of
	// "advance a live scene (uniform) by n ~ U{minSteps..maxSteps} steps"; the
	// pool is filled from the library until admission fails 50 times in a row;
	// a scene that owes nothing and has done at least its lifetime (U{lifeMin..
	// lifeMax} steps) is retired and a library scene admitted in its place.
	// Latency runs from a request's scheduled arrival to the pump observing its
	// last step.  out (16 doubles): seconds, submitted, completed, body-steps,
	// p50 / p99 latency (ms), the same for scenes of 257..512 bodies, their p50 /
	// p99 latency per requested step, live scenes, retired, admitted after the
	// start, lane steps, lanes.
	int runLoad(double duration, double rate, uint32_t minSteps, uint32_t maxSteps, uint32_t lifeMin, uint32_t lifeMax, uint64_t seed,
	            const Library& lib, double* out)
	{
		std::mt19937_64 rng(seed);
		auto uniform = [&](uint64_t lo, uint64_t hi) { return lo + rng() % (hi - lo + 1); };
		std::exponential_distribution<double> gap(rate);
		std::vector<uint32_t> live;
		std::vector<uint32_t> lifetime(scenes.size(), 0), owed(scenes.size(), 0), doneSteps(scenes.size(), 0), size(scenes.size(), 0);
		auto admitOne = [&]() -> int {
			const uint32_t k = uint32_t(uniform(0, lib.count - 1));
			const uint32_t b0 = lib.offsets[k], nb = lib.offsets[k + 1] - b0;
			uint32_t id = 0;
			const int rc = admit(nb, lib.rigid + b0, lib.types + b0, lib.geoms + 4 * size_t(b0), lib.friction + b0, 1, lib.staticPoses + 7 * size_t(k),
			                     lib.staticTypes + k, lib.staticGeoms + 4 * size_t(k), &id);
			if(rc) return rc;
			live.push_back(id);
			lifetime[id] = uint32_t(uniform(lifeMin, lifeMax));
			owed[id] = 0;
			doneSteps[id] = 0;
			size[id] = nb;
			return GBPX_OK;
		};
		for(int fails = 0; fails < 50;)
		{
			const int rc = admitOne();
			if(rc == GBPX_ERR_BUDGET) fails++;
			else if(rc) return rc;
			else fails = 0;
		}
		if(live.empty()) return GBPX_ERR_BUDGET;
		for(Lane* L : lanes) GBPX_CUDA_TRY(cudaStreamSynchronize(L->w.stream));   // admissions done
		std::vector<uint32_t> reqScene, reqSteps;
		std::vector<double> lat, lat512, perStep512;
		uint64_t tag = 0, retired = 0, admitted = 0;
		const uint64_t bodySteps0 = bodySteps, steps0 = steps;
		doneTags.clear();
		doneLatency.clear();
		const double t0 = now(), tEnd = t0 + duration;
		double tNext = t0;
		for(;;)
		{
			const double t = now();
			if(t >= tEnd) break;
			while(tNext <= t)
			{
				const uint32_t id = live[uniform(0, live.size() - 1)];
				const uint32_t n = uint32_t(uniform(minSteps, maxSteps));
				int rc = submit(id, n, tag, tNext);
				if(rc) return rc;
				reqScene.push_back(id);
				reqSteps.push_back(n);
				owed[id] += n;
				tag++;
				tNext += gap(rng);
			}
			int rc = pump(nullptr);
			if(rc) return rc;
			for(size_t i = 0; i < doneTags.size(); i++)
			{
				const uint64_t tg = doneTags[i];
				const uint32_t id = reqScene[tg], n = reqSteps[tg];
				const double l = doneLatency[i];
				lat.push_back(l);
				if(size[id] > 256 && size[id] <= 512)
				{
					lat512.push_back(l);
					perStep512.push_back(l / n);
				}
				owed[id] -= n;
				doneSteps[id] += n;
				if(owed[id] == 0 && doneSteps[id] >= lifetime[id] && live.size() > 1)
				{
					rc = retire(id);
					if(rc) return rc;
					live.erase(std::find(live.begin(), live.end(), id));
					retired++;
					rc = admitOne();
					if(rc == GBPX_OK) admitted++;
					else if(rc != GBPX_ERR_BUDGET) return rc;
				}
			}
			doneTags.clear();
			doneLatency.clear();
		}
		const double elapsed = now() - t0;
		auto pct = [](std::vector<double> v, double q) -> double {
			if(v.empty()) return -1.0;
			std::sort(v.begin(), v.end());
			const double pos = q * double(v.size() - 1);
			const size_t i = size_t(pos);
			const double f = pos - double(i);
			return 1000.0 * (i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i]);
		};
		uint64_t liveNow = 0;
		for(const auto& sc : scenes) liveNow += sc.live ? 1 : 0;
		const double vals[16] = {elapsed, double(tag), double(lat.size()), double(bodySteps - bodySteps0), pct(lat, 0.5), pct(lat, 0.99),
		                         pct(lat512, 0.5), pct(lat512, 0.99), pct(perStep512, 0.5), pct(perStep512, 0.99), double(liveNow), double(retired),
		                         double(admitted), double(steps - steps0), double(lanes.size()), 0.0};
		for(int i = 0; i < 16; i++) out[i] = vals[i];
		return GBPX_OK;
	}

	int readScene(uint32_t id, void* out)
	{
		if(id >= scenes.size() || !scenes[id].live) return GBPX_ERR_INVALID;
		const Scene& s = scenes[id];
		Lane* L = lanes[s.lane];
		GBPX_CUDA_TRY(cudaStreamSynchronize(L->w.stream));
		GBPX_CUDA_TRY(cudaMemcpy(out, L->w.bodies.ptr + L->w.hScenes[s.slot].bodyStart, size_t(s.nbBodies) * sizeof(tgs::RigidBody),
		                         cudaMemcpyDeviceToHost));
		return GBPX_OK;
	}

	void release()
	{
		for(Lane* L : lanes)
		{
			L->w.release();
			for(int i = 0; i < 2; i++)
			{
				if(L->pinned[i]) cudaFreeHost(L->pinned[i]);
				if(L->ev[i]) cudaEventDestroy(L->ev[i]);
			}
			delete L;
		}
		lanes.clear();
	}
};
} // namespace gbpx

using gbpx::Server;

// Creates a serving pool: nbClasses body-count classes, class c holding
// slots[c] slots of capacity[c] bodies and staticsPerSlot statics each.
// params/iterations as gbpx_world_create.
GBPX_API int gbpx_server_create(uint32_t nbClasses, const uint32_t* capacity, const uint32_t* slots, uint32_t staticsPerSlot, const float* params,
                                const uint32_t* iterations, uint32_t pairsPerBody, uint32_t lanesPerClass, void** outServer)
{
	if(!outServer || !nbClasses || !capacity || !slots || !params || !iterations || !iterations[0] || !iterations[1] || !pairsPerBody ||
	   !lanesPerClass)
		return GBPX_ERR_INVALID;
	for(uint32_t c = 0; c < nbClasses; c++)
		if(!capacity[c] || capacity[c] + staticsPerSlot > 65535u) return GBPX_ERR_INVALID;
	gbpx::world::StepParams sp;
	sp.dt = params[0]; sp.gx = params[1]; sp.gy = params[2]; sp.gz = params[3];
	sp.contactDistance = params[4]; sp.toleranceLength = params[5]; sp.boundsMargin = params[6];
	sp.bounceThreshold = params[7]; sp.frictionOffsetThreshold = params[8]; sp.correlationDistance = params[9]; sp.staticFriction = params[10];
	sp.persistent = params[11] != 0.0f ? 1u : 0u;
	sp.nbPos = iterations[0]; sp.nbVel = iterations[1];
	sp.largeBodies = World::DEFAULT_LARGE_BODIES;
	sp.solveVariant = gbpx::world::RESIDENT_VARIANT;
	sp.resBytes = 0;       // set at creation
	sp.resStream = World::DEFAULT_RES_STREAM;
	if(!(sp.dt > 0.0f) || !(sp.contactDistance > 0.0f)) return GBPX_ERR_INVALID;
	Server* s = new Server;
	const int rc = s->create(nbClasses, capacity, slots, staticsPerSlot, pairsPerBody, sp, lanesPerClass);
	if(rc) { s->release(); delete s; return rc; }
	*outServer = s;
	return GBPX_OK;
}

GBPX_API void gbpx_server_release(void* s)
{
	if(!s) return;
	static_cast<Server*>(s)->release();
	delete static_cast<Server*>(s);
}

// Device bytes one slot of a class takes (for sizing a pool against a memory budget).
GBPX_API uint64_t gbpx_server_slot_bytes(uint32_t capacity, uint32_t staticsPerSlot, uint32_t pairsPerBody, int persistent)
{
	return Server::slotBytes(capacity, staticsPerSlot, pairsPerBody, persistent != 0);
}

// Admits a scene (layout as one scene of gbpx_world_create) into the smallest
// free slot that holds it; GBPX_ERR_BUDGET when none is free.
GBPX_API int gbpx_server_admit(void* sv, uint32_t nbBodies, const void* rigidBodies, const int* types, const float* geoms, const float* friction,
                               uint32_t nbStatics, const float* staticPoses, const int* staticTypes, const float* staticGeoms, uint32_t* outScene)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !nbBodies || !rigidBodies || !types || !geoms || !friction || !outScene || (nbStatics && (!staticPoses || !staticTypes || !staticGeoms)))
		return GBPX_ERR_INVALID;
	for(uint32_t i = 0; i < nbBodies; i++)
		if(uint32_t(types[i]) > 3u || types[i] == 1) return GBPX_ERR_INVALID;
	return s->admit(nbBodies, rigidBodies, types, geoms, friction, nbStatics, staticPoses, staticTypes, staticGeoms, outScene);
}

// Frees a scene's slot; GBPX_ERR_STATE while it still owes requested steps.
GBPX_API int gbpx_server_retire(void* sv, uint32_t scene)
{
	Server* s = static_cast<Server*>(sv);
	return s ? s->retire(scene) : GBPX_ERR_INVALID;
}

// Queues "advance `scene` by nbSteps"; `arrival` (seconds on the server clock,
// negative = now) is the time latency is measured from.
GBPX_API int gbpx_server_submit(void* sv, uint32_t scene, uint32_t nbSteps, uint64_t tag, double arrival)
{
	Server* s = static_cast<Server*>(sv);
	return s ? s->submit(scene, nbSteps, tag, arrival) : GBPX_ERR_INVALID;
}

GBPX_API int gbpx_server_pump(void* sv, uint32_t* outIssued)
{
	Server* s = static_cast<Server*>(sv);
	return s ? s->pump(outIssued) : GBPX_ERR_INVALID;
}

// Seconds since the server was created (the clock of arrivals and latencies).
GBPX_API int gbpx_server_clock(void* sv, double* outSeconds)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !outSeconds) return GBPX_ERR_INVALID;
	*outSeconds = s->now();
	return GBPX_OK;
}

// Completed requests since the last poll: tags and latencies (seconds).
GBPX_API int gbpx_server_poll(void* sv, uint64_t* outTags, double* outLatency, uint32_t capacity, uint32_t* outCount)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !outCount) return GBPX_ERR_INVALID;
	const uint32_t n = uint32_t(std::min<size_t>(capacity, s->doneTags.size()));
	for(uint32_t i = 0; i < n; i++)
	{
		if(outTags) outTags[i] = s->doneTags[i];
		if(outLatency) outLatency[i] = s->doneLatency[i];
	}
	s->doneTags.erase(s->doneTags.begin(), s->doneTags.begin() + n);
	s->doneLatency.erase(s->doneLatency.begin(), s->doneLatency.begin() + n);
	*outCount = n;
	return GBPX_OK;
}

// Bodies of a live scene (PxRigidBodyData) after its completed steps.
GBPX_API int gbpx_server_read_scene(void* sv, uint32_t scene, void* outRigidBodies)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !outRigidBodies) return GBPX_ERR_INVALID;
	return s->readScene(scene, outRigidBodies);
}

// Snapshot of a scene that owes no steps: bodies, shapes, statics and (persistent
// mode) its pair list with each pair's contact manifold and friction patches, in
// this library's layout.  *outBytes gets the size; out (capacity bytes) the
// snapshot unless null.
GBPX_API int gbpx_server_snapshot_scene(void* sv, uint32_t scene, void* out, uint64_t capacity, uint64_t* outBytes)
{
	Server* s = static_cast<Server*>(sv);
	if(!s) return GBPX_ERR_INVALID;
	return s->snapshotScene(scene, out, capacity, outBytes);
}

// A snapshot admitted as a new scene (*outScene), continuing with the results the
// scene would have had.
GBPX_API int gbpx_server_restore_scene(void* sv, const void* snapshot, uint64_t bytes, uint32_t* outScene)
{
	Server* s = static_cast<Server*>(sv);
	if(!s) return GBPX_ERR_INVALID;
	return s->restoreScene(snapshot, bytes, outScene);
}

// out4: body-steps completed, lane steps completed, live scenes, steps in flight
GBPX_API int gbpx_server_stats(void* sv, uint64_t* out4)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !out4) return GBPX_ERR_INVALID;
	uint64_t live = 0, inflight = 0;
	for(const auto& sc : s->scenes) live += sc.live ? 1 : 0;
	for(const auto* L : s->lanes) inflight += L->nbInflight;
	out4[0] = s->bodySteps; out4[1] = s->steps; out4[2] = live; out4[3] = inflight;
	return GBPX_OK;
}

// The open-loop Poisson serving load run natively on the pool (Server::runLoad):
// the library holds nbLib scenes of one static shape each (scene k's bodies at
// libOffsets[k] .. libOffsets[k + 1]); out receives 16 figures (see runLoad).
GBPX_API int gbpx_server_run_load(void* sv, double seconds, double rate, uint32_t minSteps, uint32_t maxSteps, uint32_t lifeMin, uint32_t lifeMax,
                                  uint64_t seed, uint32_t nbLib, const uint32_t* libOffsets, const void* libRigid, const int* libTypes,
                                  const float* libGeoms, const float* libFriction, const float* libStaticPoses, const int* libStaticTypes,
                                  const float* libStaticGeoms, double* out16)
{
	Server* s = static_cast<Server*>(sv);
	if(!s || !(seconds > 0.0) || !(rate > 0.0) || !minSteps || maxSteps < minSteps || lifeMax < lifeMin || !nbLib || !libOffsets || !libRigid ||
	   !libTypes || !libGeoms || !libFriction || !libStaticPoses || !libStaticTypes || !libStaticGeoms || !out16)
		return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < nbLib; k++)
		if(libOffsets[k + 1] <= libOffsets[k]) return GBPX_ERR_INVALID;
	for(uint32_t i = 0; i < libOffsets[nbLib]; i++)
		if(uint32_t(libTypes[i]) > 3u || libTypes[i] == 1) return GBPX_ERR_INVALID;
	const Server::Library lib = {nbLib, libOffsets, static_cast<const gbpx::tgs::RigidBody*>(libRigid), libTypes, libGeoms, libFriction,
	                             libStaticPoses, libStaticTypes, libStaticGeoms};
	return s->runLoad(seconds, rate, minSteps, maxSteps, lifeMin, lifeMax, seed, lib, out16);
}
