// ORACLE (test infrastructure, never shipped): CPU restatement of the reference
// ABP broadphase's pair semantics.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load this file's library.
//
// Follows physx/source/lowlevelaabb/src/BpBroadPhaseABP.cpp:
//  * ABP::addObject/updateObject/removeObject (:3630-3710): objects store the
//    bounds given at their last add/update, inflated by their distance
//    (BoxManager::prepareData :1712-1729) -- min - d, max + d in FP32;
//  * X extents become order-preserving integer keys (BpBroadPhaseIntegerAABB.h:44
//    encodeFloat); the sweep over boxes sorted by that key reports a candidate
//    when the later box's min X does not exceed the earlier box's max X
//    (boxPruningKernel :2272, doCompleteBoxPruning_Leaf :2450); Y/Z are closed
//    float intervals (SIMD_OVERLAP_TEST_9c :2216);
//  * only pairs with at least one updated object are tested (updated vs all);
//  * groupFiltering (BpFiltering.h:90) with the LUT of BpFiltering.cpp:34;
//  * ABP_PairManager::computeCreatedDeletedPairs (:3714) for created/lost.
//
// Parity is pinned against the reference itself: tests/golden holds created/lost
// lists produced by the reference ABP on seeded inputs (see
// tests/golden/make_golden.py) and tests/test_oracle_golden.py checks this file.
#include <stdint.h>
#include <string.h>
#include <vector>
#include <algorithm>
#include <unordered_set>

#define OX extern "C" __attribute__((visibility("default")))

namespace
{
inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
inline uint32_t encodeFloat(uint32_t ir) { return (ir & 0x80000000u) ? ~ir : (ir | 0x80000000u); }

struct Box
{
	uint32_t minX, maxX;      // encoded
	float minY, minZ, maxY, maxZ;
};

struct OracleABP
{
	bool lut[7][7];
	std::vector<Box> boxes;
	std::vector<uint32_t> groups;
	std::vector<uint8_t> live;
	std::unordered_set<uint64_t> active;
	std::vector<uint32_t> createdOut, lostOut;

	OracleABP(bool discardSK, bool discardKK)
	{
		memset(lut, 0, sizeof(lut));
		auto set = [&](int a, int b, bool v) { lut[a][b] = lut[b][a] = v; };
		set(0, 2, true); set(0, 1, !discardSK); set(2, 1, true); set(2, 2, true); set(1, 1, !discardKK);
		set(0, 3, true); set(1, 3, true); set(2, 3, true); set(3, 3, true);
		set(4, 2, true); set(4, 0, true); set(4, 1, true); set(4, 4, true);
		set(5, 2, true); set(5, 0, true); set(5, 1, true); set(5, 4, true); set(5, 5, true);
		set(6, 2, true); set(6, 0, true); set(6, 1, true); set(6, 4, true); set(6, 5, true); set(6, 6, true);
	}

	bool filter(uint32_t g0, uint32_t g1) const
	{
		if(g0 == g1) return false;
		const uint32_t t0 = g0 & 7u, t1 = g1 & 7u;
		if(t0 >= 7 || t1 >= 7) return false;
		return lut[t0][t1];
	}

	void store(uint32_t id, const float* b, float d)
	{
		Box& x = boxes[id];
		const float mnx = b[0] - d, mny = b[1] - d, mnz = b[2] - d;
		const float mxx = b[3] + d, mxy = b[4] + d, mxz = b[5] + d;
		x.minX = encodeFloat(fbits(mnx));
		x.maxX = encodeFloat(fbits(mxx));
		x.minY = mny; x.minZ = mnz; x.maxY = mxy; x.maxZ = mxz;
	}

	static bool yz(const Box& a, const Box& b)
	{
		return !(b.maxY < a.minY || a.maxY < b.minY || b.maxZ < a.minZ || a.maxZ < b.minZ);
	}

	void update(const uint32_t* created, uint32_t nc, const uint32_t* updated, uint32_t nu, const uint32_t* removed, uint32_t nr,
	            const float* bounds, const uint32_t* grp, const float* dist, uint32_t cap)
	{
		if(boxes.size() < cap) { boxes.resize(cap); groups.resize(cap, 0xffffffffu); live.resize(cap, 0); }
		std::vector<uint8_t> upd(boxes.size(), 0), rem(boxes.size(), 0);
		for(uint32_t i = 0; i < nr; i++) { live[removed[i]] = 0; upd[removed[i]] = 1; rem[removed[i]] = 1; }
		for(uint32_t i = 0; i < nc; i++)
		{
			const uint32_t id = created[i];
			groups[id] = grp[id];
			store(id, bounds + 6 * size_t(id), dist[id]);
			live[id] = 1; upd[id] = 1;
		}
		for(uint32_t i = 0; i < nu; i++)
		{
			const uint32_t id = updated[i];
			store(id, bounds + 6 * size_t(id), dist[id]);
			upd[id] = 1;
		}
		// Sort live boxes by (encoded min X, handle) and sweep.
		std::vector<uint32_t> order;
		for(uint32_t i = 0; i < boxes.size(); i++) if(live[i]) order.push_back(i);
		std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
			return boxes[a].minX != boxes[b].minX ? boxes[a].minX < boxes[b].minX : a < b;
		});
		std::unordered_set<uint64_t> found;
		const size_t n = order.size();
		for(size_t i = 0; i < n; i++)
		{
			const uint32_t a = order[i];
			const Box& A = boxes[a];
			for(size_t j = i + 1; j < n; j++)
			{
				const uint32_t b = order[j];
				const Box& B = boxes[b];
				if(B.minX > A.maxX) break;
				if(!upd[a] && !upd[b]) continue;
				if(!yz(A, B)) continue;
				if(!filter(groups[a], groups[b])) continue;
				const uint32_t lo = std::min(a, b), hi = std::max(a, b);
				found.insert((uint64_t(lo) << 32) | hi);
			}
		}
		createdOut.clear();
		lostOut.clear();
		for(uint64_t k : found)
			if(!active.count(k)) { createdOut.push_back(uint32_t(k >> 32)); createdOut.push_back(uint32_t(k)); }
		std::unordered_set<uint64_t> next;
		for(uint64_t k : active)
		{
			const uint32_t id0 = uint32_t(k >> 32), id1 = uint32_t(k);
			if(!upd[id0] && !upd[id1]) { next.insert(k); continue; }
			if(found.count(k)) continue;
			if(!rem[id0] && !rem[id1]) { lostOut.push_back(id0); lostOut.push_back(id1); }
		}
		for(uint64_t k : found) next.insert(k);
		active.swap(next);
	}
};
} // namespace

OX void* orc_bp_create(int discardStaticVsKinematic, int discardKinematicVsKinematic)
{
	return new OracleABP(discardStaticVsKinematic != 0, discardKinematicVsKinematic != 0);
}

OX void orc_bp_release(void* bp) { delete static_cast<OracleABP*>(bp); }

// Same argument layout as the reference harness: bounds are 6 floats per
// handle, created/lost pairs come back as (id0, id1) with id0 < id1.
OX int orc_bp_update(void* bpv, const uint32_t* created, uint32_t nc, const uint32_t* updated, uint32_t nu, const uint32_t* removed,
                     uint32_t nr, const float* bounds, const uint32_t* groups, const float* dist, uint32_t cap, uint32_t* outCreated,
                     uint32_t maxCreated, uint32_t* nbCreated, uint32_t* outLost, uint32_t maxLost, uint32_t* nbLost)
{
	OracleABP* bp = static_cast<OracleABP*>(bpv);
	bp->update(created, nc, updated, nu, removed, nr, bounds, groups, dist, cap);
	*nbCreated = uint32_t(bp->createdOut.size() / 2);
	*nbLost = uint32_t(bp->lostOut.size() / 2);
	memcpy(outCreated, bp->createdOut.data(), sizeof(uint32_t) * 2 * std::min(*nbCreated, maxCreated));
	memcpy(outLost, bp->lostOut.data(), sizeof(uint32_t) * 2 * std::min(*nbLost, maxLost));
	return (*nbCreated <= maxCreated && *nbLost <= maxLost) ? 0 : 1;
}

OX uint32_t orc_bp_active_count(void* bpv) { return uint32_t(static_cast<OracleABP*>(bpv)->active.size()); }
