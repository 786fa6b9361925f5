// Broadphase frames written against the reference's interface
// (PxCreateBroadPhase, PxBroadPhase::update / fetchResults, PxCreateAABBManager,
// PxAABBManager::addObject / updateObject / removeObject / update /
// fetchResults, physx/include/PxBroadPhase.h), the way the reference's
// standalone-broadphase snippet drives them, linked against
// libgbpx_immediate.so.  Used by tests/test_immediate_dropin_gpu.py.
//
// stdin (binary): mode (u32: 0 = PxBroadPhase with user-managed arrays,
// 1 = PxAABBManager), frames (u32); per frame: capacity, nbCreated, nbUpdated,
// nbRemoved (u32), the created / updated / removed handles (u32), bounds
// (capacity + 1 PxBounds3), groups (capacity u32), distances (capacity f32).
// stdout (binary): per frame nbCreated, nbLost (u32), then the created and the
// lost pairs (mID0, mID1 as u32).
#include "gbpx_immediate.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace gbpx_px;

namespace
{
template <typename T> void readAll(T* p, size_t n)
{
	if(n && fread(p, sizeof(T), n, stdin) != n) { fprintf(stderr, "short input\n"); exit(2); }
}
uint32_t readU32()
{
	uint32_t v = 0;
	readAll(&v, 1);
	return v;
}
void writeResults(const PxBroadPhaseResults& r)
{
	const uint32_t counts[2] = {r.mNbCreatedPairs, r.mNbDeletedPairs};
	fwrite(counts, 4, 2, stdout);
	if(r.mNbCreatedPairs) fwrite(r.mCreatedPairs, sizeof(PxBroadPhasePair), r.mNbCreatedPairs, stdout);
	if(r.mNbDeletedPairs) fwrite(r.mDeletedPairs, sizeof(PxBroadPhasePair), r.mNbDeletedPairs, stdout);
}
} // namespace

int main()
{
	const uint32_t mode = readU32(), frames = readU32();
	PxBroadPhaseDesc desc(PxBroadPhaseType::eABP);
	PxBroadPhase* bp = PxCreateBroadPhase(desc);
	if(!bp) { fprintf(stderr, "PxCreateBroadPhase failed\n"); return 1; }
	if(bp->getType() != PxBroadPhaseType::eABP || bp->getRegions() != nullptr) return 1;
	PxAABBManager* manager = mode == 1 ? PxCreateAABBManager(*bp) : nullptr;
	if(mode == 1 && (!manager || PxCreateAABBManager(*bp) != nullptr)) { fprintf(stderr, "PxCreateAABBManager failed\n"); return 1; }
	PxAllocatorCallback* allocator = bp->getAllocator();
	PxBounds3* bounds = nullptr;
	PxBpFilterGroup* groups = nullptr;
	float* distances = nullptr;
	uint32_t cap = 0;
	std::vector<PxBounds3> inBounds;
	std::vector<PxBpFilterGroup> inGroups;
	std::vector<float> inDist;
	for(uint32_t f = 0; f < frames; f++)
	{
		const uint32_t capacity = readU32(), nc = readU32(), nu = readU32(), nr = readU32();
		std::vector<PxBpIndex> created(nc), updated(nu), removed(nr);
		readAll(created.data(), nc);
		readAll(updated.data(), nu);
		readAll(removed.data(), nr);
		inBounds.resize(capacity + 1);
		inGroups.resize(capacity);
		inDist.resize(capacity);
		readAll(inBounds.data(), capacity + 1);
		readAll(inGroups.data(), capacity);
		readAll(inDist.data(), capacity);
		PxBroadPhaseResults results;
		if(mode == 0)
		{
			// the user's persistent arrays, from the broadphase's allocator
			if(capacity > cap)
			{
				allocator->deallocate(bounds);
				allocator->deallocate(groups);
				allocator->deallocate(distances);
				bounds = static_cast<PxBounds3*>(allocator->allocate(sizeof(PxBounds3) * (capacity + 1), "bounds", __FILE__, __LINE__));
				groups = static_cast<PxBpFilterGroup*>(allocator->allocate(sizeof(PxBpFilterGroup) * capacity, "groups", __FILE__, __LINE__));
				distances = static_cast<float*>(allocator->allocate(sizeof(float) * capacity, "distances", __FILE__, __LINE__));
				cap = capacity;
			}
			memcpy(bounds, inBounds.data(), sizeof(PxBounds3) * (capacity + 1));
			memcpy(groups, inGroups.data(), sizeof(PxBpFilterGroup) * capacity);
			memcpy(distances, inDist.data(), sizeof(float) * capacity);
			const PxBroadPhaseUpdateData data(created.data(), nc, updated.data(), nu, removed.data(), nr, bounds, groups, distances, capacity);
			bp->updateAndFetchResults(results, data);
		}
		else
		{
			for(PxBpIndex i : removed) manager->removeObject(i);
			for(PxBpIndex i : created) manager->addObject(i, inBounds[i], inGroups[i], inDist[i]);
			for(PxBpIndex i : updated) manager->updateObject(i, &inBounds[i], &inDist[i]);
			manager->updateAndFetchResults(results);
		}
		writeResults(results);
	}
	if(manager) manager->release();
	allocator->deallocate(bounds);
	allocator->deallocate(groups);
	allocator->deallocate(distances);
	bp->release();
	return 0;
}
