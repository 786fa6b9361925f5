// Constraint batching rule of PxBatchConstraintsTGS, host side.
//
// Follows the reference's partitioning (physx/source/lowleveldynamics/src/
// DyConstraintPartition.cpp:476 classifyConstraintDesc, :571 writeConstraintDesc,
// :858 partitionContactConstraints) and header creation
// (physx/source/immediatemode/src/NpImmediateMode.cpp:159 createHeaders):
//  * dynamic-dynamic constraints, in input order, take the lowest partition bit
//    free in both bodies' 32-bit masks; when none is free they overflow into the
//    next round of 32 partitions;
//  * a dynamic-static constraint goes into partition maxDynamicPartition(body)
//    + k, the k-th static constraint of that body, so statics come after all of
//    the body's dynamic constraints, one per partition;
//  * headers group up to 4 consecutive constraints of one partition.
// The order it produces is what makes a partition a set of body-disjoint
// constraints that the GPU solves as one parallel wave.
#pragma once
#include <stdint.h>
#include <vector>
#include <algorithm>

namespace gbpx
{
namespace batching
{
struct Result
{
	std::vector<uint32_t> order;          // ordered constraint indices
	std::vector<uint32_t> partitionEnds;  // end offset (exclusive) of each partition in `order`
	std::vector<uint32_t> headerStart, headerStride;
};

// kind (may be null: one kind): per constraint its PxSolverConstraintDesc
// constraint type; a header only joins consecutive constraints of one kind
// (createHeaders, physx/source/immediatemode/src/NpImmediateMode.cpp:159).
inline void partition(const uint32_t* bodyA, const uint32_t* bodyB, uint32_t n, uint32_t nbDyn, Result& out, const uint8_t* kind = nullptr)
{
	const uint32_t MAXP = 32;
	std::vector<uint32_t> progress(nbDyn, 0), maxNormal(nbDyn, 0), maxStatic(nbDyn, 0);
	std::vector<uint32_t> perPartition(MAXP, 0);
	std::vector<uint32_t> overflow;
	auto take = [&](uint32_t a, uint32_t b, uint32_t& part) {
		const uint32_t mask = ~progress[a] & ~progress[b];
		if(!mask) return false;
		part = uint32_t(__builtin_ctz(mask));
		progress[a] |= 1u << part;
		progress[b] |= 1u << part;
		return true;
	};
	for(uint32_t i = 0; i < n; i++)
	{
		const bool aA = bodyA[i] < nbDyn, aB = bodyB[i] < nbDyn;
		if(aA && aB)
		{
			uint32_t part;
			if(!take(bodyA[i], bodyB[i], part)) { overflow.push_back(i); continue; }
			perPartition[part]++;
			maxNormal[bodyA[i]] = std::max(maxNormal[bodyA[i]], part + 1);
			maxNormal[bodyB[i]] = std::max(maxNormal[bodyB[i]], part + 1);
		}
		else
		{
			if(aA) maxStatic[bodyA[i]]++;
			if(aB) maxStatic[bodyB[i]]++;
		}
	}
	uint32_t start = 0;
	std::vector<uint32_t> pending = overflow;
	while(!pending.empty())
	{
		std::fill(progress.begin(), progress.end(), 0u);
		start += MAXP;
		perPartition.resize(perPartition.size() + MAXP, 0);
		std::vector<uint32_t> next;
		for(uint32_t i : pending)
		{
			uint32_t part;
			if(!take(bodyA[i], bodyB[i], part)) { next.push_back(i); continue; }
			perPartition[start + part]++;
			maxNormal[bodyA[i]] = std::max(maxNormal[bodyA[i]], start + part + 1);
			maxNormal[bodyB[i]] = std::max(maxNormal[bodyB[i]], start + part + 1);
		}
		pending.swap(next);
	}
	for(uint32_t b = 0; b < nbDyn; b++)
	{
		const uint32_t need = maxNormal[b] + maxStatic[b];
		if(need > perPartition.size()) perPartition.resize(need, 0);
		for(uint32_t k = 0; k < maxStatic[b]; k++) perPartition[maxNormal[b] + k]++;
	}
	uint32_t acc = 0;
	for(uint32_t& c : perPartition) { const uint32_t t = c; c = acc; acc += t; }
	std::fill(progress.begin(), progress.end(), 0u);
	std::vector<uint32_t> staticProgress(nbDyn, 0);
	out.order.assign(n, 0xffffffffu);
	std::vector<uint32_t> ov;
	for(uint32_t i = 0; i < n; i++)
	{
		const bool aA = bodyA[i] < nbDyn, aB = bodyB[i] < nbDyn;
		if(aA && aB)
		{
			uint32_t part;
			if(!take(bodyA[i], bodyB[i], part)) { ov.push_back(i); continue; }
			out.order[perPartition[part]++] = i;
		}
		else if(aA || aB)
		{
			const uint32_t b = aA ? bodyA[i] : bodyB[i];
			out.order[perPartition[maxNormal[b] + staticProgress[b]++]++] = i;
		}
	}
	start = 0;
	while(!ov.empty())
	{
		std::fill(progress.begin(), progress.end(), 0u);
		start += MAXP;
		std::vector<uint32_t> next;
		for(uint32_t i : ov)
		{
			uint32_t part;
			if(!take(bodyA[i], bodyB[i], part)) { next.push_back(i); continue; }
			out.order[perPartition[start + part]++] = i;
		}
		ov.swap(next);
	}
	out.partitionEnds = perPartition;
	uint32_t maxPartition = 0, prev = 0;
	for(size_t a = 0; a < perPartition.size(); a++, maxPartition++)
	{
		if(perPartition[a] == prev) break;
		prev = perPartition[a];
	}
	out.headerStart.clear();
	out.headerStride.clear();
	uint32_t cur = 0;
	uint32_t maxJ = n == 0 ? 0 : perPartition[0];
	for(uint32_t a = 0; a < n;)
	{
		out.headerStart.push_back(a);
		const uint32_t loopMax = std::min(maxJ - a, 4u);
		uint32_t j = 0;
		if(loopMax > 0)
		{
			j = 1;
			if(cur < maxPartition)
			{
				if(!kind) j = loopMax;
				else
				{
					// (a constraint between two non-dynamic bodies is not placed: its slot stays unset)
					const uint32_t first = out.order[a];
					while(j < loopMax && first < n && out.order[a + j] < n && kind[out.order[a + j]] == kind[first]) j++;
				}
			}
		}
		out.headerStride.push_back(j);
		if(maxJ == a + j && maxJ != n)
		{
			cur++;
			maxJ = perPartition[cur];
		}
		a += j;
	}
}
} // namespace batching
} // namespace gbpx
