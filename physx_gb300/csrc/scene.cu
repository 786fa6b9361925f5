// Large-scene rigid-body step for the GB300: ONE scene of up to millions of
// bodies, each stage spread over the whole GPU (the batched world in world.cu
// gives every scene one warp, which suits scenes of up to a few thousand
// bodies).  The frame is the reference immediate-mode snippet's
// (physx/snippets/snippetimmediatemode/SnippetImmediateMode.cpp:473
// stepPhysics), persistent pair state included (:657-676, :941-978):
//   1. bounds of every dynamic body plus the margin feed the ABP broadphase of
//      gbpx_bp (radix-sorted sweep, statics created once and never moved); its
//      active set is every overlapping pair, sorted by (id0, id1), statics
//      numbered after the dynamic bodies;
//   2. narrowphase: pairs queued by kind, one kernel per kind, a thread per
//      pair; in persistent mode a pair finds its slot in last frame's pair list
//      by binary search and carries its PCM manifold (double-buffered);
//   3. constraints = pairs with contacts, in pair order; PxBatchConstraintsTGS
//      runs on the host (batching.h: the rule is sequential in constraint order);
//   4. solver bodies, contact rows (a thread per constraint, last frame's
//      friction patches correlated), TGS position/velocity iterations partition
//      by partition (a thread per constraint of one partition, the partition's
//      constraints touch disjoint bodies), integration after every position
//      iteration, PxIntegrateSolverBodiesTGS and write-back.
// Arithmetic is the world's: the same device functions, the same order.
#include "common.cuh"
#include <optional>
#include "contacts.cuh"
#include "solver.cuh"
#include "step_common.cuh"
#include "batching.h"
#include "bp_internal.h"
#include "radix_sort.cuh"
#include <vector>

GBPX_API int gbpx_bp_create(int discardStaticVsKinematic, int discardKinematicVsKinematic, void** outBp);
GBPX_API void gbpx_bp_release(void* bp);
GBPX_API int gbpx_bp_update(void* bp, const uint32_t* created, uint32_t nbCreated, const uint32_t* updated, uint32_t nbUpdated,
                            const uint32_t* removed, uint32_t nbRemoved, const float* bounds, const uint32_t* groups, const float* distances,
                            uint32_t capacity);
GBPX_API int gbpx_bp_fetch_results(void* bp, const uint32_t** created, uint32_t* nbCreated, const uint32_t** lost, uint32_t* nbLost);

namespace gbpx
{
namespace scene
{
using world::NB_KINDS;
using world::NO_PREV;
using world::StepParams;

// Device view of one large scene.
struct SceneDev
{
	uint32_t nbDyn, nbStatic;
	tgs::RigidBody* bodies;
	const int* types;
	const float4* geoms;
	const float* friction;
	const int* staticTypes;
	const float4* staticGeoms;
	const float* staticPose;   // 7 floats per static (PxTransform)
};

__device__ __forceinline__ void shapeOf(const SceneDev& s, uint32_t id, int& type, float g[4], Tr& pose)
{
	if(id < s.nbDyn)
	{
		type = s.types[id];
		const float4 gg = s.geoms[id];
		g[0] = gg.x; g[1] = gg.y; g[2] = gg.z; g[3] = gg.w;
		const tgs::RigidBody& rb = s.bodies[id];
		pose.q.x = rb.q[0]; pose.q.y = rb.q[1]; pose.q.z = rb.q[2]; pose.q.w = rb.q[3];
		pose.p = v3(rb.p[0], rb.p[1], rb.p[2]);
	}
	else
	{
		const uint32_t k = id - s.nbDyn;
		type = s.staticTypes[k];
		const float4 gg = s.staticGeoms[k];
		g[0] = gg.x; g[1] = gg.y; g[2] = gg.z; g[3] = gg.w;
		pose = world::loadStaticPose(s.staticPose + 7 * size_t(k));
	}
}

// Bounds of shapes [0, count) (dynamic bodies, then statics) plus the margin
// (6 floats: min xyz, max xyz), the world broadphase's arithmetic; planes are
// unbounded.
__global__ void boundsKernel(SceneDev s, uint32_t count, float margin, float* __restrict__ out)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= count) return;
	int type;
	float g[4];
	Tr pose;
	shapeOf(s, i, type, g, pose);
	V3 mn, mx;
	world::shapeBounds(type, make_float4(g[0], g[1], g[2], g[3]), pose, mn, mx);
	float* o = out + 6 * size_t(i);
	o[0] = mn.x - margin; o[1] = mn.y - margin; o[2] = mn.z - margin;
	o[3] = mx.x + margin; o[4] = mx.y + margin; o[5] = mx.z + margin;
}

// Pair kinds: each active pair is queued under its kind (queue order does not
// matter: every output is written to the pair's own slot).
__global__ void kindKernel(SceneDev s, const unsigned long long* __restrict__ keys, uint32_t nbPairs, uint32_t* __restrict__ queue,
                           uint32_t queueCap, uint32_t* __restrict__ kindCount)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t lane = threadIdx.x & 31;
	uint32_t kind = NB_KINDS;
	if(k < nbPairs)
	{
		const unsigned long long key = keys[k];
		const uint32_t i = uint32_t(key >> 32), j = uint32_t(key);
		const int ti = i < s.nbDyn ? s.types[i] : s.staticTypes[i - s.nbDyn];
		const int tj = j < s.nbDyn ? s.types[j] : s.staticTypes[j - s.nbDyn];
		kind = world::kindOf(ti, tj);
	}
	// one atomic per kind present in the warp
	for(uint32_t t = 0; t < NB_KINDS; t++)
	{
		const uint32_t peers = __ballot_sync(0xffffffffu, kind == t);
		if(!peers) continue;
		const uint32_t leader = __ffs(peers) - 1;
		uint32_t base = 0;
		if(lane == leader) base = atomicAdd(&kindCount[t], uint32_t(__popc(peers)));
		base = __shfl_sync(0xffffffffu, base, leader);
		if(kind == t) queue[size_t(t) * queueCap + base + __popc(peers & laneMaskLt())] = k;
	}
}

// Narrowphase of one pair kind: a thread per queued pair (grid-stride).
template <int TA, int TB>
__global__ void __launch_bounds__(128) narrowphaseKernel(SceneDev s, StepParams sp, const unsigned long long* __restrict__ keys,
                                                         const unsigned long long* __restrict__ keysPrev, uint32_t nbPrev,
                                                         const uint32_t* __restrict__ queue, const uint32_t* __restrict__ kindCount,
                                                         uint32_t* __restrict__ prevSlot, const np::ManifoldRecord* __restrict__ manifoldsIn,
                                                         np::ManifoldRecord* __restrict__ manifoldsOut, tgs::FrictionState* __restrict__ frictionOut,
                                                         float4* __restrict__ contacts, uint32_t* __restrict__ contactCount)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	constexpr uint32_t KIND = TA == 0 ? uint32_t(TB) : (TA == 1 ? uint32_t(TB + 2) : (TA == 2 ? uint32_t(TB + 4) : 8u));
	constexpr bool CACHED = world::cachedPairKind(KIND);
	const uint32_t count = kindCount[KIND];
	for(uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x)
	{
		const uint32_t k = queue[q];
		const unsigned long long key = keys[k];
		const uint32_t i = uint32_t(key >> 32), j = uint32_t(key);
		uint32_t prev = NO_PREV;
		if(sp.persistent)
		{
			uint32_t lo = 0, hi = nbPrev;
			while(lo < hi)
			{
				const uint32_t mid = (lo + hi) >> 1;
				if(keysPrev[mid] < key) lo = mid + 1;
				else hi = mid;
			}
			if(lo < nbPrev && keysPrev[lo] == key) prev = lo;
			prevSlot[k] = prev;
		}
		int ta, tb;
		float ga[4], gb[4];
		Tr pa, pb;
		shapeOf(s, i, ta, ga, pa);
		shapeOf(s, j, tb, gb, pb);
		const bool swap = ta > tb;
		np::Buffer buf;
		np::Manifold m;
		if(CACHED && sp.persistent && prev != NO_PREV) np::loadManifold(manifoldsIn[prev], m);
		if(swap) world::generateKind<TA, TB>(gb, ga, pb, pa, sp, m, buf);
		else world::generateKind<TA, TB>(ga, gb, pa, pb, sp, m, buf);
		if(sp.persistent)
		{
			if(CACHED) np::storeManifold(m, manifoldsOut[k]);
			frictionOut[k].count = 0;   // the row preparation writes a constraint's patches
		}
		float4* o = contacts + size_t(k) * 8;
		for(int c = 0; c < buf.count; c++)
		{
			V3 nn = buf.c[c].n;
			if(swap) nn = neg(nn);
			o[2 * c] = make_float4(nn.x, nn.y, nn.z, buf.c[c].sep);
			o[2 * c + 1] = make_float4(buf.c[c].p.x, buf.c[c].p.y, buf.c[c].p.z, 0.0f);
		}
		contactCount[k] = uint32_t(buf.count);
	}
}

using NpKernel = void (*)(SceneDev, StepParams, const unsigned long long*, const unsigned long long*, uint32_t, const uint32_t*, const uint32_t*,
                          uint32_t*, const np::ManifoldRecord*, np::ManifoldRecord*, tgs::FrictionState*, float4*, uint32_t*);
static const NpKernel* npKernels()
{
	static const NpKernel k[NB_KINDS] = {narrowphaseKernel<0, 0>, narrowphaseKernel<0, 1>, narrowphaseKernel<0, 2>,
	                                     narrowphaseKernel<0, 3>, narrowphaseKernel<1, 2>, narrowphaseKernel<1, 3>,
	                                     narrowphaseKernel<2, 2>, narrowphaseKernel<2, 3>, narrowphaseKernel<3, 3>};
	return k;
}

// Constraints = pairs with contacts, in pair order (stable compaction).
// Also totals the contacts (totalContacts, one atomic per warp).
__global__ void countConstraintsKernel(const uint32_t* __restrict__ contactCount, uint32_t n, uint32_t* __restrict__ blockCounts,
                                       unsigned long long* __restrict__ totalContacts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t cnt = k < n ? contactCount[k] : 0u;
	const uint32_t c = __syncthreads_count(cnt > 0);
	if(threadIdx.x == 0) blockCounts[blockIdx.x] = c;
	for(int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
	if((threadIdx.x & 31) == 0 && cnt) atomicAdd(totalContacts, (unsigned long long)cnt);
}

__global__ void emitConstraintsKernel(const uint32_t* __restrict__ contactCount, const unsigned long long* __restrict__ keys, uint32_t n,
                                      const uint32_t* __restrict__ blockOffsets, uint32_t* __restrict__ consPair, uint32_t* __restrict__ consA,
                                      uint32_t* __restrict__ consB)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	__shared__ uint32_t warpCounts[32];
	const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
	const bool v = k < n && contactCount[k] > 0;
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint32_t ballot = __ballot_sync(0xffffffffu, v);
	if(lane == 0) warpCounts[warp] = __popc(ballot);
	__syncthreads();
	if(warp == 0)
	{
		const uint32_t nw = blockDim.x >> 5;
		const uint32_t c = lane < nw ? warpCounts[lane] : 0u;
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
		const uint32_t r = blockOffsets[blockIdx.x] + warpCounts[warp] + __popc(ballot & laneMaskLt());
		const unsigned long long key = keys[k];
		consPair[r] = k;
		consA[r] = uint32_t(key >> 32);
		consB[r] = uint32_t(key);
	}
}

// ------------------------------------------------------------------ device batching
// PxBatchConstraintsTGS's rule (DyConstraintPartition.cpp:858, restated in
// batching.h) reproduced exactly in parallel.  The rule colours the
// dynamic-dynamic constraints greedily in input order: a constraint takes the
// lowest partition bit free in both bodies' masks, which holds the bits of the
// earlier constraints of those bodies.  So a constraint's partition depends only
// on the earlier constraints that share a body with it, and it can be computed
// as soon as those are done (the parallel greedy colouring of Jones and
// Plassmann, with input order as the priority): each pass colours every
// constraint whose predecessors in both bodies' lists finished in earlier
// passes.  At most one constraint per body is ready in a pass (the first
// unfinished one of its list), so body masks are never written concurrently.
// The number of passes is the longest chain of constraints linked through
// shared bodies in input order (tens on contact graphs).  A constraint that
// finds all 32 bits taken would go to the rule's next round of partitions: that
// rare case is left to the host path.  Static constraints then take partition
// maxDynamicPartition(body) + their rank among the body's static constraints,
// and a stable sort by partition gives the reference's placement order.
namespace sbatch
{
constexpr uint32_t NONE = 0xffffffffu;
constexpr uint32_t NOT_DONE = 0xffffffffu;
constexpr uint32_t DEFERRED = 0xffffu;

// Two incidence entries per constraint, in constraint order: (body, c) for each
// dynamic body of a dynamic-dynamic constraint; (nbDyn + body, c) for the
// dynamic body of a static constraint, whose second entry sorts last.
__global__ void incidenceKernel(const uint32_t* __restrict__ consA, const uint32_t* __restrict__ consB, uint32_t nc, uint32_t nbDyn,
                                uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t* __restrict__ ddList, uint32_t* __restrict__ counts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if(c >= nc) return;
	const uint32_t a = consA[c], b = consB[c];
	const bool dd = a < nbDyn && b < nbDyn;
	keys[2 * c] = dd ? a : nbDyn + (a < nbDyn ? a : b);
	keys[2 * c + 1] = dd ? b : NONE;
	vals[2 * c] = c;
	vals[2 * c + 1] = c;
	if(dd) ddList[atomicAdd(&counts[0], 1u)] = c;
}

// Each constraint's predecessor in each of its bodies' lists (dynamic-dynamic
// constraints), and where each body's list of static constraints starts.
__global__ void linkKernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n, uint32_t nbDyn,
                           const uint32_t* __restrict__ consA, uint32_t* __restrict__ prevOf, uint32_t* __restrict__ staticRunStart)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= n) return;
	const uint32_t key = keys[e];
	if(key == NONE) return;
	const bool runStart = e == 0 || keys[e - 1] != key;
	if(key < nbDyn)
	{
		const uint32_t c = vals[e];
		prevOf[2 * c + (key == consA[c] ? 0u : 1u)] = runStart ? NONE : vals[e - 1];
	}
	else if(runStart)
		staticRunStart[key - nbDyn] = e;
}

// One pass of the colouring.  donePass[c] is the pass that coloured c.
__global__ void colorPassKernel(const uint32_t* __restrict__ ddList, uint32_t nDD, const uint32_t* __restrict__ consA,
                                const uint32_t* __restrict__ consB, const uint32_t* __restrict__ prevOf, uint32_t* __restrict__ donePass,
                                uint32_t* __restrict__ part, uint32_t* __restrict__ mask, uint32_t* __restrict__ maxNormal, uint32_t pass,
                                uint32_t* __restrict__ counts)
{
	gridDependencyWait();   // launched dependent on the previous pass (launchDependent)
	gridLaunchDependents();
	uint32_t done = 0;
	for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nDD; i += gridDim.x * blockDim.x)
	{
		const uint32_t c = ddList[i];
		if(donePass[c] != NOT_DONE) continue;
		const uint32_t pa = prevOf[2 * c], pb = prevOf[2 * c + 1];
		if((pa != NONE && donePass[pa] >= pass) || (pb != NONE && donePass[pb] >= pass)) continue;
		const uint32_t a = consA[c], b = consB[c];
		const uint32_t freeBits = ~mask[a] & ~mask[b];
		if(freeBits)
		{
			const uint32_t p = uint32_t(__ffs(freeBits)) - 1u;
			mask[a] |= 1u << p;
			mask[b] |= 1u << p;
			maxNormal[a] = max(maxNormal[a], p + 1u);
			maxNormal[b] = max(maxNormal[b], p + 1u);
			part[c] = p;
		}
		else
		{
			part[c] = DEFERRED;
			counts[2] = 1u;   // the rule's next round: the host path takes this step
		}
		donePass[c] = pass;
		done++;
	}
	for(int o = 16; o > 0; o >>= 1) done += __shfl_xor_sync(0xffffffffu, done, o);
	if((threadIdx.x & 31) == 0 && done) atomicSub(&counts[1], done);
}

// Partition of the static constraints, partition counts, sort keys.
__global__ void staticPartKernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n, uint32_t nbDyn,
                                 const uint32_t* __restrict__ staticRunStart, const uint32_t* __restrict__ maxNormal, uint32_t* __restrict__ part)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= n) return;
	const uint32_t key = keys[e];
	if(key == NONE || key < nbDyn) return;
	const uint32_t body = key - nbDyn;
	part[vals[e]] = maxNormal[body] + (e - staticRunStart[body]);
}

constexpr uint32_t MAX_PARTS = 4096;
__global__ void partKeysKernel(const uint32_t* __restrict__ part, uint32_t nc, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                               uint32_t* __restrict__ perPart, uint32_t* __restrict__ counts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
	if(c >= nc) return;
	const uint32_t p = part[c];
	keys[c] = p;
	vals[c] = c;
	if(p < MAX_PARTS) atomicAdd(&perPart[p], 1u);
	atomicMax(&counts[3], p + 1u);
}

// Inclusive scan of the partition counts into end offsets (one block).
__global__ void partEndsKernel(uint32_t* __restrict__ perPart, const uint32_t* __restrict__ counts)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	if(threadIdx.x != 0) return;
	const uint32_t np = min(counts[3], MAX_PARTS);
	uint32_t acc = 0;
	for(uint32_t p = 0; p < np; p++) { acc += perPart[p]; perPart[p] = acc; }
}
} // namespace sbatch

// Solver bodies (PxConstructSolverBodiesTGS / PxConstructStaticSolverBodyTGS).
__global__ void bodiesKernel(SceneDev s, StepParams sp, tgs::BodyVel* __restrict__ vel, tgs::BodyTx* __restrict__ tx, tgs::BodyData* __restrict__ data,
                             Tr* __restrict__ pose)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < s.nbDyn)
	{
		Tr p;
		tgs::constructDynamicBody(s.bodies[i], v3(sp.gx, sp.gy, sp.gz), sp.dt, vel[i], tx[i], data[i], p);
		pose[i] = p;
	}
	else if(i < s.nbDyn + s.nbStatic)
	{
		const Tr p = world::loadStaticPose(s.staticPose + 7 * size_t(i - s.nbDyn));
		tgs::constructStaticBody(p, vel[i], tx[i], data[i]);
		pose[i] = p;
	}
}

// Contact rows of the constraint at solve position r (PxCreateContactConstraintsTGS
// for one descriptor).  order[r] indexes the constraint list; headers are runs of
// up to 4 constraints of one partition, and full runs of 4 take the block path.
__global__ void prepKernel(SceneDev s, StepParams sp, uint32_t nc, const uint32_t* __restrict__ order, const uint32_t* __restrict__ consPair,
                           const uint32_t* __restrict__ partEnds, uint32_t nbPart, const unsigned long long* __restrict__ keys,
                           const float4* __restrict__ contacts, const uint32_t* __restrict__ contactCount, const tgs::BodyVel* __restrict__ vel,
                           const tgs::BodyTx* __restrict__ tx, const tgs::BodyData* __restrict__ data, const Tr* __restrict__ pose,
                           const uint32_t* __restrict__ prevSlot, const tgs::FrictionState* __restrict__ frictionIn,
                           tgs::FrictionState* __restrict__ frictionOut, uint32_t* __restrict__ orderedPair, tgs::ConstraintRecord* __restrict__ recs)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= nc) return;
	uint32_t lo = 0, hi = nbPart - 1;   // partition of r: first end above r
	while(lo < hi)
	{
		const uint32_t mid = (lo + hi) >> 1;
		if(partEnds[mid] > r) hi = mid;
		else lo = mid + 1;
	}
	const uint32_t start = lo ? partEnds[lo - 1] : 0u, size = partEnds[lo] - start;
	const bool block = (r - start) < (size & ~3u);
	const uint32_t k = consPair[order[r]];
	orderedPair[r] = k;
	const unsigned long long key = keys[k];
	const uint32_t a = uint32_t(key >> 32), b = uint32_t(key);
	const uint32_t n = s.nbDyn;
	const float fa = s.friction[a];
	const float fb = b < n ? s.friction[b] : sp.staticFriction;
	const float mu = (fa + fb) * 0.5f;
	tgs::Contact cs[tgs::MAX_CONTACTS];
	const uint32_t cnt = contactCount[k];
	const float4* src = contacts + size_t(k) * 8;
	for(uint32_t c = 0; c < cnt; c++)
	{
		const float4 nn = src[2 * c], p4 = src[2 * c + 1];
		cs[c].n = v3(nn.x, nn.y, nn.z);
		cs[c].sep = nn.w;
		cs[c].p = v3(p4.x, p4.y, p4.z);
		cs[c].staticFriction = mu;
		cs[c].dynamicFriction = mu;
		cs[c].restitution = 0.0f;
	}
	const tgs::PrepParams pp = world::prepParams(sp);
	const tgs::FrictionState* prevFriction = nullptr;
	tgs::FrictionState* written = nullptr;
	if(sp.persistent)
	{
		const uint32_t prev = prevSlot[k];
		if(prev != NO_PREV) prevFriction = frictionIn + prev;
		written = frictionOut + k;
	}
	if(block)
		tgs::prepConstraintBlock(cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, b < n, b == 0,
		                         recs[r], prevFriction, written);
	else
		tgs::prepConstraint(cs, int(cnt), int(a), int(b), vel[a], vel[b], tx[a], tx[b], data[a], data[b], pose[a], pose[b], pp, recs[r],
		                    prevFriction, written);
}

// One partition of one iteration: a thread per constraint (the partition's
// constraints touch disjoint dynamic bodies).  The last iteration of a
// persistent step marks the friction patches whose friction was clamped.
__global__ void solvePartitionKernel(tgs::ConstraintRecord* __restrict__ recs, uint32_t begin, uint32_t end, tgs::BodyVel* __restrict__ vel,
                                     uint32_t nbDyn, float minPen, float elapsed, const uint32_t* __restrict__ orderedPair,
                                     tgs::FrictionState* __restrict__ frictionOut)
{
	// launched dependent on the previous partition / integration (launchDependent)
	gridDependencyWait();
	gridLaunchDependents();
	const uint32_t r = begin + blockIdx.x * blockDim.x + threadIdx.x;
	if(r >= end) return;
	tgs::ConstraintRecord& rec = recs[r];
	if(rec.nbPatches == 0) return;
	const uint32_t a = uint32_t(rec.bodyA), b = uint32_t(rec.bodyB);
	tgs::BodyVel b0 = vel[a];
	tgs::BodyVel b1 = vel[b];
	const bool dynB = b < nbDyn;
	uint32_t broken = 0;
	tgs::solveRecord(rec, b0, b1, dynB, minPen, elapsed, frictionOut ? &broken : nullptr);
	if(broken)
	{
		tgs::FrictionState& fs = frictionOut[orderedPair[r]];
		tgs::ConstraintRecord* group[4] = {nullptr, nullptr, nullptr, nullptr};
		if(rec.isBlock())
		{
			const uint32_t r0 = begin + ((r - begin) & ~3u);
			for(uint32_t l = 0; l < 4; l++) group[l] = recs + r0 + l;
		}
		for(int pi = 0; pi < rec.nbPatches; pi++)
			if(broken & (1u << pi))
			{
				const int slotIdx = rec.isBlock() ? tgs::blockBrokenSlot(group, pi) : pi;
				if(uint32_t(slotIdx) < fs.count) fs.patches[slotIdx].broken = 1;
			}
	}
	vel[a].lin = b0.lin;
	vel[a].ang = b0.ang;
	if(dynB)
	{
		vel[b].lin = b1.lin;
		vel[b].ang = b1.ang;
	}
}

__global__ void integrateKernel(tgs::BodyVel* __restrict__ vel, tgs::BodyTx* __restrict__ tx, uint32_t nbDyn, float stepDt)
{
	gridDependencyWait();   // launched dependent on the last partition (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= nbDyn) return;
	tgs::BodyVel v = vel[i];
	tgs::integrateStep(v, tx[i], stepDt);
	vel[i].dLin = v.dLin;
	vel[i].dAng = v.dAng;
}

// PxIntegrateSolverBodiesTGS and write-back into the PxRigidBodyData records.
__global__ void finalizeKernel(SceneDev s, const tgs::BodyVel* __restrict__ vel, const tgs::BodyTx* __restrict__ tx, const Tr* __restrict__ pose)
{
	gridDependencyWait();   // may be launched dependent on the previous kernel (launchDependent)
	gridLaunchDependents();
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= s.nbDyn) return;
	tgs::BodyVel v = vel[i];
	Tr p = pose[i];
	V3 wv;
	tgs::finalizeBody(v, tx[i], p, wv);
	tgs::RigidBody& rb = s.bodies[i];
	rb.linVel[0] = v.lin.x; rb.linVel[1] = v.lin.y; rb.linVel[2] = v.lin.z;
	rb.angVel[0] = wv.x; rb.angVel[1] = wv.y; rb.angVel[2] = wv.z;
	rb.q[0] = p.q.x; rb.q[1] = p.q.y; rb.q[2] = p.q.z; rb.q[3] = p.q.w;
	rb.p[0] = p.p.x; rb.p[1] = p.p.y; rb.p[2] = p.p.z;
}

// One large scene resident on the device.
struct Scene
{
	static constexpr uint32_t STAGES = 6;   // bounds + broadphase, narrowphase, constraints + batching, bodies + rows, iterations, write-back
	SceneDev dev() { return SceneDev{nbDyn, nbStatic, bodies.ptr, types.ptr, geoms.ptr, frictionCoef.ptr, staticTypes.ptr, staticGeoms.ptr, staticPose.ptr}; }

	uint32_t nbDyn = 0, nbStatic = 0;
	StepParams sp{};
	void* bp = nullptr;
	cudaStream_t stream = 0;   // the broadphase's stream carries the whole step
	DevBuf<tgs::RigidBody> bodies;
	DevBuf<int> types, staticTypes;
	DevBuf<float4> geoms, staticGeoms;
	DevBuf<float> frictionCoef, staticPose, bounds;
	DevBuf<unsigned long long> keysPrev, totalContacts;
	DevBuf<uint32_t> queue, kindCount, prevSlot, contactCount, blockCounts, consPair, consA, consB, order, partEnds, orderedPair;
	DevBuf<float4> contacts;
	DevBuf<np::ManifoldRecord> manifolds[2];
	DevBuf<tgs::FrictionState> frictionState[2];
	DevBuf<tgs::BodyVel> vel;
	DevBuf<tgs::BodyTx> tx;
	DevBuf<tgs::BodyData> data;
	DevBuf<Tr> pose;
	DevBuf<tgs::ConstraintRecord> recs;
	// device batching: incidence lists, predecessors, colouring state
	DevBuf<uint32_t> incKeys, incVals, incKeysAlt, incValsAlt, sortHist, ddList, prevOf, donePass, partOf, bodyMask, maxNormal, staticRunStart,
	    perPart, batchCounts;
	HostBuf<uint32_t> hBatch;   // counts and partition ends read back
	std::vector<uint32_t> hPartEnds;
	uint32_t lastColorPasses = 0;
	bool deviceBatchEnabled = true;   // false: PxBatchConstraintsTGS's rule always on the host (comparison path)
	bool lastBatchOnDevice = false;
	HostBuf<uint32_t> hConsA, hConsB, hOrder, hSmall;
	HostBuf<unsigned long long> hTotal;
	uint32_t parity = 0, nbPairs = 0, nbPrev = 0, nbConstraints = 0, nbPartitions = 0;
	uint64_t nbContacts = 0;
	bool havePrev = false;
	size_t pairCap = 0;
	cudaEvent_t ev[STAGES + 1] = {};
	double stageAcc[STAGES] = {};
	uint32_t timedSteps = 0;
	bool timing = false;

	int create(uint32_t n, const void* rigid, const int* t, const float* g, const float* mu, uint32_t m, const float* sPose, const int* sTypes,
	           const float* sGeoms, const float* params, const uint32_t* iterations)
	{
		nbDyn = n;
		nbStatic = m;
		sp.dt = params[0]; sp.gx = params[1]; sp.gy = params[2]; sp.gz = params[3];
		sp.contactDistance = params[4]; sp.toleranceLength = params[5]; sp.boundsMargin = params[6];
		sp.bounceThreshold = params[7]; sp.frictionOffsetThreshold = params[8]; sp.correlationDistance = params[9];
		sp.staticFriction = params[10];
		sp.persistent = params[11] != 0.0f ? 1u : 0u;
		sp.nbPos = iterations[0];
		sp.nbVel = iterations[1];
		int rc = gbpx_bp_create(0, 0, &bp);
		if(rc) return rc;
		stream = bpi::stream(bp);
		const uint32_t total = n + m;
		if(bodies.reserve(n) || types.reserve(n) || geoms.reserve(n) || frictionCoef.reserve(n) || staticTypes.reserve(m + 1) ||
		   staticGeoms.reserve(m + 1) || staticPose.reserve(7 * size_t(m) + 1) || bounds.reserve(6 * size_t(total)) || kindCount.reserve(NB_KINDS) ||
		   totalContacts.reserve(1) || vel.reserve(total) || tx.reserve(total) || data.reserve(total) || pose.reserve(total) ||
		   hSmall.reserve(16) || hTotal.reserve(1) || bodyMask.reserve(n + 1) || maxNormal.reserve(n + 1) || staticRunStart.reserve(n + 1) ||
		   perPart.reserve(sbatch::MAX_PARTS) || batchCounts.reserve(4) || hBatch.reserve(4 + sbatch::MAX_PARTS))
			return GBPX_ERR_NOMEM;
		GBPX_CUDA_TRY(cudaMemcpyAsync(bodies.ptr, rigid, size_t(n) * sizeof(tgs::RigidBody), cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(types.ptr, t, size_t(n) * 4, cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(geoms.ptr, g, size_t(n) * 16, cudaMemcpyHostToDevice, stream));
		GBPX_CUDA_TRY(cudaMemcpyAsync(frictionCoef.ptr, mu, size_t(n) * 4, cudaMemcpyHostToDevice, stream));
		if(m)
		{
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticTypes.ptr, sTypes, size_t(m) * 4, cudaMemcpyHostToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticGeoms.ptr, sGeoms, size_t(m) * 16, cudaMemcpyHostToDevice, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(staticPose.ptr, sPose, size_t(m) * 28, cudaMemcpyHostToDevice, stream));
		}
		for(uint32_t k = 0; k <= STAGES; k++) GBPX_CUDA_TRY(cudaEventCreate(&ev[k]));
		// every shape enters the broadphase once: dynamic bodies in their own filter
		// groups, statics in the static group (PxBpFilterGroup encodings)
		(void)launchDependent(boundsKernel, divUp(total, 128), 128, stream, dev(), total, sp.boundsMargin, bounds.ptr);
		GBPX_CUDA_TRY(cudaGetLastError());
		std::vector<float> hb(6 * size_t(total));
		GBPX_CUDA_TRY(cudaMemcpyAsync(hb.data(), bounds.ptr, hb.size() * 4, cudaMemcpyDeviceToHost, stream));
		GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
		std::vector<uint32_t> ids(total), groups(total);
		std::vector<float> dist(total, 0.0f);
		for(uint32_t i = 0; i < total; i++)
		{
			ids[i] = i;
			groups[i] = i < n ? (((i + 1u) << 3) | 2u) : 0u;
		}
		rc = gbpx_bp_update(bp, ids.data(), total, nullptr, 0, nullptr, 0, hb.data(), groups.data(), dist.data(), total);
		if(rc) return rc;
		const uint32_t *c0, *c1;
		uint32_t nc0, nc1;
		return gbpx_bp_fetch_results(bp, &c0, &nc0, &c1, &nc1);
	}

	void release()
	{
		if(stream) cudaStreamSynchronize(stream);
		for(auto& e : ev)
			if(e) cudaEventDestroy(e);
		bodies.release(); types.release(); staticTypes.release(); geoms.release(); staticGeoms.release(); frictionCoef.release();
		staticPose.release(); bounds.release(); keysPrev.release(); totalContacts.release(); queue.release(); kindCount.release();
		prevSlot.release(); contactCount.release(); blockCounts.release(); consPair.release(); consA.release(); consB.release(); order.release();
		partEnds.release(); orderedPair.release(); contacts.release(); vel.release(); tx.release(); data.release(); pose.release();
		recs.release(); hConsA.release(); hConsB.release(); hOrder.release(); hSmall.release(); hTotal.release();
		incKeys.release(); incVals.release(); incKeysAlt.release(); incValsAlt.release(); sortHist.release(); ddList.release(); prevOf.release();
		donePass.release(); partOf.release(); bodyMask.release(); maxNormal.release(); staticRunStart.release(); perPart.release();
		batchCounts.release(); hBatch.release();
		for(int k = 0; k < 2; k++) { manifolds[k].release(); frictionState[k].release(); }
		if(bp) gbpx_bp_release(bp);
		bp = nullptr;
		stream = 0;
	}

	// Per-pair buffers for `need` pairs; the state of last frame's pairs survives.
	int reservePairs(uint32_t need)
	{
		if(need <= pairCap) return GBPX_OK;
		const size_t cap = std::max<size_t>(need + need / 4, 1024);
		if(queue.reserve(size_t(NB_KINDS) * cap) || prevSlot.reserve(cap) || contactCount.reserve(cap) || blockCounts.reserve(cap / 256 + 2) ||
		   consPair.reserve(cap) || consA.reserve(cap) || consB.reserve(cap) || order.reserve(cap) || partEnds.reserve(cap) ||
		   orderedPair.reserve(cap) || contacts.reserve(8 * cap) || recs.reserve(cap) || hConsA.reserve(cap) || hConsB.reserve(cap) ||
		   hOrder.reserve(cap) || incKeys.reserve(2 * cap) || incVals.reserve(2 * cap) || incKeysAlt.reserve(2 * cap) ||
		   incValsAlt.reserve(2 * cap) || sortHist.reserve(radixSortHistEntries(uint32_t(2 * cap))) || ddList.reserve(cap) ||
		   prevOf.reserve(2 * cap) || donePass.reserve(cap) || partOf.reserve(cap))
			return GBPX_ERR_NOMEM;
		if(sp.persistent)
		{
			const uint32_t p = parity;
			if(manifolds[p].reserve(cap, stream, true, nbPrev) || frictionState[p].reserve(cap, stream, true, nbPrev) ||
			   manifolds[p ^ 1u].reserve(cap) || frictionState[p ^ 1u].reserve(cap) || keysPrev.reserve(cap, stream, true, nbPrev))
				return GBPX_ERR_NOMEM;
		}
		pairCap = cap;
		return GBPX_OK;
	}

	// host-side profiler zone of the stage in progress (closed by the next mark)
	std::optional<Zone> stageZone;
	void mark(uint32_t k)
	{
		static const char* const names[STAGES] = {"gbpx::scene::broadphase", "gbpx::scene::narrowphase", "gbpx::scene::batching",
		                                          "gbpx::scene::rows", "gbpx::scene::iterations", "gbpx::scene::writeBack"};
		if(timing) cudaEventRecord(ev[k], stream);
		stageZone.reset();
		if(k < STAGES) stageZone.emplace(names[k]);
	}

	// PxBatchConstraintsTGS for the nc constraints (consA, consB) on the device
	// (sbatch): fills order, partEnds and hPartEnds.  Returns false, with nothing
	// filled, when a constraint needs the rule's second round of partitions (the
	// caller then batches on the host).
	int deviceBatch(uint32_t nc, bool& done)
	{
		done = false;
		const cudaStream_t s = stream;
		const uint32_t n2 = 2 * nc;
		GBPX_CUDA_TRY(cudaMemsetAsync(batchCounts.ptr, 0, 16, s));
		(void)launchDependent(sbatch::incidenceKernel, divUp(nc, 256), 256, s, consA.ptr, consB.ptr, nc, nbDyn, incKeys.ptr, incVals.ptr, ddList.ptr,
		                                                       batchCounts.ptr);
		GBPX_CUDA_TRY(cudaMemsetAsync(bodyMask.ptr, 0, size_t(nbDyn) * 4, s));
		GBPX_CUDA_TRY(cudaMemsetAsync(maxNormal.ptr, 0, size_t(nbDyn) * 4, s));
		GBPX_CUDA_TRY(cudaMemsetAsync(donePass.ptr, 0xff, size_t(nc) * 4, s));
		GBPX_CUDA_TRY(cudaMemsetAsync(perPart.ptr, 0, sbatch::MAX_PARTS * 4, s));
		// stable sort of the incidence entries by list (body, then static lists): bits for 2 nbDyn list keys
		int bits = 1;
		while(bits < 32 && (1ull << bits) <= 2ull * nbDyn) bits++;
		const int endBit = std::min(32, (bits + 7) / 8 * 8 + (bits % 8 ? 0 : 0));
		const bool alt = radixSort<uint32_t, true>(incKeys.ptr, incVals.ptr, incKeysAlt.ptr, incValsAlt.ptr, n2, 0, endBit, sortHist.ptr, s);
		const uint32_t* sk = alt ? incKeysAlt.ptr : incKeys.ptr;
		const uint32_t* sv = alt ? incValsAlt.ptr : incVals.ptr;
		(void)launchDependent(sbatch::linkKernel, divUp(n2, 256), 256, s, sk, sv, n2, nbDyn, consA.ptr, prevOf.ptr, staticRunStart.ptr);
		// remaining = number of dynamic-dynamic constraints
		GBPX_CUDA_TRY(cudaMemcpyAsync(batchCounts.ptr + 1, batchCounts.ptr, 4, cudaMemcpyDeviceToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(hBatch.ptr, batchCounts.ptr, 16, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaStreamSynchronize(s));
		const uint32_t nDD = hBatch.ptr[0];
		const uint32_t grid = std::max(1u, std::min(divUp(nDD, 256), 152u * 8u));
		uint32_t pass = 0;
		while(nDD)
		{
			// a pass always colours the first unfinished constraint, so nDD passes always suffice
			for(int k = 0; k < 8; k++)
				GBPX_CUDA_TRY(launchDependent(sbatch::colorPassKernel, grid, 256, s, ddList.ptr, nDD, consA.ptr, consB.ptr, prevOf.ptr, donePass.ptr,
				                              partOf.ptr, bodyMask.ptr, maxNormal.ptr, ++pass, batchCounts.ptr));
			GBPX_CUDA_TRY(cudaGetLastError());
			GBPX_CUDA_TRY(cudaMemcpyAsync(hBatch.ptr, batchCounts.ptr, 16, cudaMemcpyDeviceToHost, s));
			GBPX_CUDA_TRY(cudaStreamSynchronize(s));
			if(hBatch.ptr[1] == 0 || pass > nDD + 8) break;
		}
		lastColorPasses = pass;
		if(nDD && (hBatch.ptr[1] != 0 || hBatch.ptr[2] != 0)) return GBPX_OK;   // second round needed: host path
		(void)launchDependent(sbatch::staticPartKernel, divUp(n2, 256), 256, s, sk, sv, n2, nbDyn, staticRunStart.ptr, maxNormal.ptr, partOf.ptr);
		// stable sort by partition: the reference's placement (input order within a partition)
		(void)launchDependent(sbatch::partKeysKernel, divUp(nc, 256), 256, s, partOf.ptr, nc, incKeys.ptr, incVals.ptr, perPart.ptr, batchCounts.ptr);
		(void)launchDependent(sbatch::partEndsKernel, 1, 32, s, perPart.ptr, batchCounts.ptr);
		const bool alt2 = radixSort<uint32_t, true>(incKeys.ptr, incVals.ptr, incKeysAlt.ptr, incValsAlt.ptr, nc, 0, 16, sortHist.ptr, s);
		GBPX_CUDA_TRY(cudaMemcpyAsync(order.ptr, alt2 ? incValsAlt.ptr : incVals.ptr, size_t(nc) * 4, cudaMemcpyDeviceToDevice, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(hBatch.ptr, batchCounts.ptr, 16, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaMemcpyAsync(hBatch.ptr + 4, perPart.ptr, sbatch::MAX_PARTS * 4, cudaMemcpyDeviceToHost, s));
		GBPX_CUDA_TRY(cudaStreamSynchronize(s));
		const uint32_t nbParts = hBatch.ptr[3];
		if(nbParts > sbatch::MAX_PARTS) return GBPX_OK;   // (never on contact scenes) host path
		hPartEnds.assign(hBatch.ptr + 4, hBatch.ptr + 4 + nbParts);
		GBPX_CUDA_TRY(cudaMemcpyAsync(partEnds.ptr, perPart.ptr, size_t(nbParts) * 4, cudaMemcpyDeviceToDevice, s));
		done = true;
		return GBPX_OK;
	}

	int step()
	{
		struct CloseZone { std::optional<Zone>& z; ~CloseZone() { z.reset(); } } closeZone{stageZone};
		const SceneDev d = dev();
		mark(0);
		// 1. bounds + broadphase; last frame's pair list is kept for the slot lookup
		if(sp.persistent && havePrev && nbPairs)
		{
			uint32_t cnt = 0;
			const unsigned long long* cur = bpi::activePairs(bp, &cnt);
			if(keysPrev.reserve(std::max<size_t>(cnt, pairCap), stream, false)) return GBPX_ERR_NOMEM;
			GBPX_CUDA_TRY(cudaMemcpyAsync(keysPrev.ptr, cur, size_t(cnt) * 8, cudaMemcpyDeviceToDevice, stream));
			nbPrev = cnt;
		}
		else
			nbPrev = 0;
		(void)launchDependent(boundsKernel, divUp(nbDyn, 128), 128, stream, d, nbDyn, sp.boundsMargin, bounds.ptr);
		GBPX_CUDA_TRY(cudaGetLastError());
		int rc = bpi::updateFromDevice(bp, bounds.ptr, nbDyn);
		if(rc) return rc;
		const unsigned long long* keys = bpi::activePairs(bp, &nbPairs);
		rc = reservePairs(nbPairs ? nbPairs : 1);
		if(rc) return rc;
		mark(1);
		// 2. narrowphase
		const uint32_t par = parity;
		GBPX_CUDA_TRY(cudaMemsetAsync(kindCount.ptr, 0, NB_KINDS * 4, stream));
		GBPX_CUDA_TRY(cudaMemsetAsync(totalContacts.ptr, 0, 8, stream));
		if(nbPairs)
		{
			(void)launchDependent(kindKernel, divUp(nbPairs, 128), 128, stream, d, keys, nbPairs, queue.ptr, uint32_t(pairCap), kindCount.ptr);
			const uint32_t grid = std::min<uint32_t>(divUp(nbPairs, 128), 152u * 16u);
			for(uint32_t k = 0; k < NB_KINDS; k++)
				(void)launchDependent(npKernels()[k], grid, 128, stream, d, sp, keys, keysPrev.ptr, nbPrev, queue.ptr + size_t(k) * pairCap, kindCount.ptr, prevSlot.ptr,
				                                         manifolds[par].ptr, manifolds[par ^ 1u].ptr, frictionState[par ^ 1u].ptr, contacts.ptr,
				                                         contactCount.ptr);
			GBPX_CUDA_TRY(cudaGetLastError());
		}
		mark(2);
		// 3. constraints (pairs with contacts, pair order) and PxBatchConstraintsTGS on the host
		nbConstraints = 0;
		if(nbPairs)
		{
			const uint32_t nb = divUp(nbPairs, 256);
			(void)launchDependent(countConstraintsKernel, nb, 256, stream, contactCount.ptr, nbPairs, blockCounts.ptr, totalContacts.ptr);
			GBPX_CUDA_TRY(cudaMemsetAsync(blockCounts.ptr + nb, 0, 4, stream));
			(void)launchDependent(rs::scanKernel, 1, 1024, stream, blockCounts.ptr, nb + 1);
			(void)launchDependent(emitConstraintsKernel, nb, 256, stream, contactCount.ptr, keys, nbPairs, blockCounts.ptr, consPair.ptr, consA.ptr, consB.ptr);
			GBPX_CUDA_TRY(cudaGetLastError());
			GBPX_CUDA_TRY(cudaMemcpyAsync(hSmall.ptr, blockCounts.ptr + nb, 4, cudaMemcpyDeviceToHost, stream));
			GBPX_CUDA_TRY(cudaMemcpyAsync(hTotal.ptr, totalContacts.ptr, 8, cudaMemcpyDeviceToHost, stream));
			GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
			nbConstraints = hSmall.ptr[0];
			nbContacts = hTotal.ptr[0];
		}
		const uint32_t nc = nbConstraints;
		hPartEnds.clear();
		lastBatchOnDevice = false;
		if(nc)
		{
			bool onDevice = false;
			if(deviceBatchEnabled)
			{
				rc = deviceBatch(nc, onDevice);
				if(rc) return rc;
			}
			lastBatchOnDevice = onDevice;
			if(!onDevice)
			{
				// the rule's second round of partitions (a body in more than 32 constraints): on the host
				batching::Result batch;
				GBPX_CUDA_TRY(cudaMemcpyAsync(hConsA.ptr, consA.ptr, size_t(nc) * 4, cudaMemcpyDeviceToHost, stream));
				GBPX_CUDA_TRY(cudaMemcpyAsync(hConsB.ptr, consB.ptr, size_t(nc) * 4, cudaMemcpyDeviceToHost, stream));
				GBPX_CUDA_TRY(cudaStreamSynchronize(stream));
				batching::partition(hConsA.ptr, hConsB.ptr, nc, nbDyn, batch);
				memcpy(hOrder.ptr, batch.order.data(), size_t(nc) * 4);
				GBPX_CUDA_TRY(cudaMemcpyAsync(order.ptr, hOrder.ptr, size_t(nc) * 4, cudaMemcpyHostToDevice, stream));
				GBPX_CUDA_TRY(cudaMemcpyAsync(partEnds.ptr, batch.partitionEnds.data(), batch.partitionEnds.size() * 4, cudaMemcpyHostToDevice, stream));
				GBPX_CUDA_TRY(cudaStreamSynchronize(stream));   // the host vector goes out of scope
				hPartEnds = batch.partitionEnds;
				// the rule sizes its table in rounds of 32: drop the empty partitions at the end
				while(hPartEnds.size() > 1 && hPartEnds.back() == hPartEnds[hPartEnds.size() - 2]) hPartEnds.pop_back();
			}
		}
		nbPartitions = uint32_t(hPartEnds.size());
		mark(3);
		// 4. solver bodies and contact rows
		(void)launchDependent(bodiesKernel, divUp(nbDyn + nbStatic, 128), 128, stream, d, sp, vel.ptr, tx.ptr, data.ptr, pose.ptr);
		if(nc)
			(void)launchDependent(prepKernel, divUp(nc, 128), 128, stream, d, sp, nc, order.ptr, consPair.ptr, partEnds.ptr, nbPartitions, keys, contacts.ptr,
			                                               contactCount.ptr, vel.ptr, tx.ptr, data.ptr, pose.ptr, prevSlot.ptr, frictionState[par].ptr,
			                                               frictionState[par ^ 1u].ptr, orderedPair.ptr, recs.ptr);
		GBPX_CUDA_TRY(cudaGetLastError());
		mark(4);
		// 5. iterations, partition by partition
		const float stepDt = sp.dt / float(sp.nbPos);
		float elapsed = 0.0f;
		for(uint32_t it = 0; it < sp.nbPos + sp.nbVel; it++)
		{
			const bool posIter = it < sp.nbPos;
			const bool last = it + 1 == sp.nbPos + sp.nbVel;
			const float minPen = posIter ? -FLT_MAX : 0.0f;
			tgs::FrictionState* broken = sp.persistent && last ? frictionState[par ^ 1u].ptr : nullptr;
			for(uint32_t p = 0; p < nbPartitions; p++)
			{
				const uint32_t b = p ? hPartEnds[p - 1] : 0u, e = hPartEnds[p];
				// each launch overlaps the previous kernel's tail and waits on the device
				// for its completion (programmatic dependent launch)
				if(e > b)
					GBPX_CUDA_TRY(launchDependent(solvePartitionKernel, divUp(e - b, 128), 128, stream, recs.ptr, b, e, vel.ptr, nbDyn, minPen, elapsed,
					                              orderedPair.ptr, broken));
			}
			if(posIter)
			{
				GBPX_CUDA_TRY(launchDependent(integrateKernel, divUp(nbDyn, 128), 128, stream, vel.ptr, tx.ptr, nbDyn, stepDt));
				elapsed += stepDt;
			}
		}
		GBPX_CUDA_TRY(cudaGetLastError());
		mark(5);
		// 6. PxIntegrateSolverBodiesTGS + write-back
		(void)launchDependent(finalizeKernel, divUp(nbDyn, 128), 128, stream, d, vel.ptr, tx.ptr, pose.ptr);
		GBPX_CUDA_TRY(cudaGetLastError());
		mark(6);
		if(sp.persistent) parity ^= 1u;
		havePrev = true;
		return GBPX_OK;
	}

	int timeSteps(uint32_t n, float* outMs)
	{
		timing = true;
		for(uint32_t k = 0; k < STAGES; k++) stageAcc[k] = 0.0;
		double total = 0.0;
		for(uint32_t s = 0; s < n; s++)
		{
			const int rc = step();
			if(rc) { timing = false; return rc; }
			GBPX_CUDA_TRY(cudaEventSynchronize(ev[STAGES]));
			for(uint32_t k = 0; k < STAGES; k++)
			{
				float ms = 0.0f;
				GBPX_CUDA_TRY(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
				stageAcc[k] += ms;
				total += ms;
			}
		}
		timing = false;
		outMs[0] = float(total / n);
		for(uint32_t k = 0; k < STAGES; k++) outMs[1 + k] = float(stageAcc[k] / n);
		return GBPX_OK;
	}
};
} // namespace scene
} // namespace gbpx

using gbpx::scene::Scene;

// One large scene (the reference snippet's frame over one scene of any size,
// each stage spread over the whole GPU).  Layout as one scene of
// gbpx_world_create: rigidBodies PxRigidBodyData[nbDyn]; types, geoms (4
// floats), friction per dynamic body; static poses (PxTransform), types, geoms;
// params (12 floats) and iterations (pos, vel) as gbpx_world_create.
GBPX_API int gbpx_scene_create(uint32_t nbDyn, const void* rigidBodies, const int* types, const float* geoms, const float* friction,
                               uint32_t nbStatic, const float* staticPoses, const int* staticTypes, const float* staticGeoms, const float* params,
                               const uint32_t* iterations, void** outScene)
{
	if(!outScene || !nbDyn || !rigidBodies || !types || !geoms || !friction || !params || !iterations) return GBPX_ERR_INVALID;
	if(nbStatic && (!staticPoses || !staticTypes || !staticGeoms)) return GBPX_ERR_INVALID;
	if(!(params[0] > 0.0f) || !iterations[0] || !iterations[1] || uint64_t(nbDyn) + nbStatic >= 0xffffffffull) return GBPX_ERR_INVALID;
	for(uint32_t i = 0; i < nbDyn; i++)
		if(types[i] != 0 && types[i] != 2 && types[i] != 3) return GBPX_ERR_INVALID;   // dynamic: sphere, capsule, box
	for(uint32_t i = 0; i < nbStatic; i++)
		if(staticTypes[i] < 0 || staticTypes[i] > 3) return GBPX_ERR_INVALID;
	Scene* s = new Scene;
	const int rc = s->create(nbDyn, rigidBodies, types, geoms, friction, nbStatic, staticPoses, staticTypes, staticGeoms, params, iterations);
	if(rc)
	{
		s->release();
		delete s;
		return rc;
	}
	*outScene = s;
	return GBPX_OK;
}

GBPX_API void gbpx_scene_release(void* sv)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s) return;
	s->release();
	delete s;
}

// Advances the scene by nbSteps frames (returns when the last has finished).
GBPX_API int gbpx_scene_step(void* sv, uint32_t nbSteps)
{
	gbpx::Zone zone("gbpx::scene::step");
	Scene* s = static_cast<Scene*>(sv);
	if(!s) return GBPX_ERR_INVALID;
	for(uint32_t k = 0; k < nbSteps; k++)
	{
		const int rc = s->step();
		if(rc) return rc;
	}
	GBPX_CUDA_TRY(cudaStreamSynchronize(s->stream));
	return GBPX_OK;
}

GBPX_API int gbpx_scene_get_bodies(void* sv, void* outRigid)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !outRigid) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(outRigid, s->bodies.ptr, size_t(s->nbDyn) * sizeof(gbpx::tgs::RigidBody), cudaMemcpyDeviceToHost, s->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s->stream));
	return GBPX_OK;
}

GBPX_API int gbpx_scene_set_bodies(void* sv, const void* rigid)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !rigid) return GBPX_ERR_INVALID;
	GBPX_CUDA_TRY(cudaMemcpyAsync(s->bodies.ptr, rigid, size_t(s->nbDyn) * sizeof(gbpx::tgs::RigidBody), cudaMemcpyHostToDevice, s->stream));
	GBPX_CUDA_TRY(cudaStreamSynchronize(s->stream));
	return GBPX_OK;
}

// out4: pairs, constraints (pairs with contacts), contacts, partitions of the last step.
GBPX_API int gbpx_scene_stats(void* sv, uint64_t* out4)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !out4) return GBPX_ERR_INVALID;
	out4[0] = s->nbPairs; out4[1] = s->nbConstraints; out4[2] = s->nbContacts; out4[3] = s->nbPartitions;
	return GBPX_OK;
}

// PxBatchConstraintsTGS on the device (1, the default) or on the host (0).  The
// two give the same order and partitions; the device form falls back to the
// host for a frame in which a body has more than 32 dynamic constraints.
GBPX_API int gbpx_scene_set_device_batching(void* sv, int enable)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s) return GBPX_ERR_INVALID;
	s->deviceBatchEnabled = enable != 0;
	return GBPX_OK;
}

// Batching of the last frame: out2[0] = colouring passes of the device
// batching, out2[1] = 1 when the frame was batched on the device.
GBPX_API int gbpx_scene_batch_info(void* sv, uint32_t* out2)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !out2) return GBPX_ERR_INVALID;
	out2[0] = s->lastColorPasses;
	out2[1] = s->lastBatchOnDevice ? 1u : 0u;
	return GBPX_OK;
}

// Runs nbSteps frames with CUDA events on the scene's stream between the
// stages; outMs[0] = average milliseconds per frame, outMs[1..6] = average per
// stage: bounds + broadphase, narrowphase, constraint list + batching,
// solver bodies + rows, iterations, write-back.  Host work inside a frame
// (the broadphase's count read-backs, the batching) is inside the times.
GBPX_API int gbpx_scene_time_steps(void* sv, uint32_t nbSteps, float* outMs)
{
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !nbSteps || !outMs) return GBPX_ERR_INVALID;
	return s->timeSteps(nbSteps, outMs);
}

// End to end through host memory: uploads the bodies from rigidIn (host
// PxRigidBodyData), advances nbSteps frames, downloads them into rigidOut;
// outMs = event-timed milliseconds of the whole call on the scene's stream.
GBPX_API int gbpx_scene_step_host(void* sv, const void* rigidIn, void* rigidOut, uint32_t nbSteps, float* outMs)
{
	gbpx::Zone zone("gbpx::scene::stepHost");
	Scene* s = static_cast<Scene*>(sv);
	if(!s || !rigidIn || !rigidOut || !outMs) return GBPX_ERR_INVALID;
	const size_t bytes = size_t(s->nbDyn) * sizeof(gbpx::tgs::RigidBody);
	GBPX_CUDA_TRY(cudaEventRecord(s->ev[0], s->stream));
	GBPX_CUDA_TRY(cudaMemcpyAsync(s->bodies.ptr, rigidIn, bytes, cudaMemcpyHostToDevice, s->stream));
	for(uint32_t k = 0; k < nbSteps; k++)
	{
		const int rc = s->step();
		if(rc) return rc;
	}
	GBPX_CUDA_TRY(cudaMemcpyAsync(rigidOut, s->bodies.ptr, bytes, cudaMemcpyDeviceToHost, s->stream));
	GBPX_CUDA_TRY(cudaEventRecord(s->ev[Scene::STAGES], s->stream));
	GBPX_CUDA_TRY(cudaEventSynchronize(s->ev[Scene::STAGES]));
	GBPX_CUDA_TRY(cudaEventElapsedTime(outMs, s->ev[0], s->ev[Scene::STAGES]));
	return GBPX_OK;
}
