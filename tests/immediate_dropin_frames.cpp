// Frames of one scene written against the reference's interface
// (physx::immediate: PxGenerateContacts, PxConstructSolverBodiesTGS,
// PxConstructStaticSolverBodyTGS, PxBatchConstraintsTGS,
// PxCreateContactConstraintsTGS, PxSolveConstraintsTGS,
// PxIntegrateSolverBodiesTGS) the way the reference's immediate-mode snippet
// drives it in its persistent mode, linked against libgbpx_immediate.so.  Used
// by tests/test_immediate_dropin_gpu.py.
//
// Every frame: shape bounds (+ margin), every overlapping pair in (id0, id1)
// order, contacts with the pair's PxCache, one contact constraint per pair with
// contacts carrying the pair's friction data from the last frame, batching, the
// TGS solve and integration, bodies written back.  A pair keeps its cache and
// friction data while its bounds overlap, loses its friction data when it has
// no contact (SnippetImmediateMode.cpp:657-676, 941-978).
//
// stdin (binary): nbDyn, nbStatic, nbFrames (u32); PxRigidBodyData[nbDyn];
// dynamic types (i32) and geometry (4 floats) per body, friction per body;
// static poses (PxTransform), types and geometry; params: dt, gravity xyz,
// contactDistance, toleranceLength, boundsMargin, bounceThreshold,
// frictionOffsetThreshold, correlationDistance, staticFriction (11 floats).
// stdout (binary): per frame the PxRigidBodyData array after the frame and the
// frame's constraint count (u32).
#include "gbpx_immediate.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

using namespace gbpx_px;

namespace
{
template <typename T> void readAll(T* p, size_t n)
{
	if(n && fread(p, sizeof(T), n, stdin) != n) { fprintf(stderr, "short input\n"); exit(2); }
}

struct Shape
{
	union { PxGeometry any; PxSphereGeometry sphere; PxCapsuleGeometry capsule; PxBoxGeometry box; PxPlaneGeometry plane; };
	Shape() { memset(this, 0, sizeof(*this)); }
	void set(int type, const float* g)
	{
		any.mType = type;
		if(type == 0) sphere.radius = g[0];
		if(type == 2) { capsule.radius = g[0]; capsule.halfHeight = g[1]; }
		if(type == 3) box.halfExtents = PxVec3{g[0], g[1], g[2]};
	}
};

struct Recorder : PxContactRecorder
{
	std::vector<std::vector<PxContactPoint>> perPair;
	bool recordContacts(const PxContactPoint* cp, uint32_t n, uint32_t index) override
	{
		perPair[index].assign(cp, cp + n);
		return true;
	}
};

// memory that lives two frames (caches and friction data of one frame are read the next)
struct TwoFrameArena
{
	std::vector<void*> blocks[2];
	int frame = 0;
	uint8_t* alloc(uint32_t bytes)
	{
		void* p = nullptr;
		if(posix_memalign(&p, 16, bytes ? bytes : 16)) return nullptr;
		blocks[frame & 1].push_back(p);
		return static_cast<uint8_t*>(p);
	}
	void nextFrame()
	{
		frame++;
		for(void* p : blocks[frame & 1]) free(p);
		blocks[frame & 1].clear();
	}
	~TwoFrameArena()
	{
		for(auto& b : blocks)
			for(void* p : b) free(p);
	}
};

struct CacheAllocator : PxCacheAllocator
{
	TwoFrameArena arena;
	uint8_t* allocateCacheData(const uint32_t byteSize) override { return arena.alloc(byteSize); }
};

struct ConstraintAllocator : PxConstraintAllocator
{
	TwoFrameArena rows, friction;
	uint8_t* reserveConstraintData(const uint32_t byteSize) override { return rows.alloc(byteSize); }
	uint8_t* reserveFrictionData(const uint32_t byteSize) override { return friction.alloc(byteSize); }
};

struct PairState
{
	PxCache cache;
	uint8_t* friction = nullptr;
	uint32_t nbFriction = 0;
	PairState() { memset(&cache, 0, sizeof(cache)); }
};

// shape bounds: sphere r; capsule |axis| * halfHeight + r; box sum of |columns| * extents (column-form rotation)
void shapeBounds(int type, const float* g, const PxTransform& t, float margin, float* out)
{
	const float qx = t.q.x, qy = t.q.y, qz = t.q.z, qw = t.q.w;
	float e[3];
	if(type == 0) { e[0] = e[1] = e[2] = g[0]; }
	else if(type == 2)
	{
		const float x2 = qx * 2.0f, w2 = qw * 2.0f;
		const float ax = (qw * w2 + qx * x2) - 1.0f, ay = qz * w2 + qy * x2, az = (-qy) * w2 + qz * x2;
		e[0] = fabsf(ax) * g[1] + g[0]; e[1] = fabsf(ay) * g[1] + g[0]; e[2] = fabsf(az) * g[1] + g[0];
	}
	else if(type == 3)
	{
		const float x2 = qx + qx, y2 = qy + qy, z2 = qz + qz, w2 = qw + qw;
		const float cx = x2 * qw, cy = y2 * qw, cz = z2 * qw, cw = w2 * qw + (-1.0f);
		const float c0[3] = {qx * x2 + cw, qy * x2 + cz, qz * x2 + (-cy)};
		const float c1[3] = {qx * y2 + (-cz), qy * y2 + cw, qz * y2 + cx};
		const float c2[3] = {qx * z2 + cy, qy * z2 + (-cx), qz * z2 + cw};
		for(int k = 0; k < 3; k++) e[k] = (fabsf(c0[k]) * g[0] + fabsf(c1[k]) * g[1]) + fabsf(c2[k]) * g[2];
	}
	else
	{
		for(int k = 0; k < 3; k++) { out[k] = -1e30f - margin; out[3 + k] = 1e30f + margin; }
		return;
	}
	const float p[3] = {t.p.x, t.p.y, t.p.z};
	for(int k = 0; k < 3; k++) { out[k] = (p[k] - e[k]) - margin; out[3 + k] = (p[k] + e[k]) + margin; }
}

uint32_t encodeFloat(float f)
{
	uint32_t u;
	memcpy(&u, &f, 4);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

bool overlap(const float* a, const float* b)
{
	if(encodeFloat(b[0]) > encodeFloat(a[3]) || encodeFloat(a[0]) > encodeFloat(b[3])) return false;
	return !(b[4] < a[1] || a[4] < b[1] || b[5] < a[2] || a[5] < b[2]);
}
} // namespace

int main()
{
	uint32_t hdr[3];
	readAll(hdr, 3);
	const uint32_t nbDyn = hdr[0], nbStatic = hdr[1], nbFrames = hdr[2];
	std::vector<PxRigidBodyData> rigid(nbDyn);
	readAll(rigid.data(), nbDyn);
	std::vector<int> types(nbDyn), staticTypes(nbStatic);
	std::vector<float> geoms(4 * size_t(nbDyn)), frictionOf(nbDyn), staticGeoms(4 * size_t(nbStatic));
	std::vector<PxTransform> staticPoses(nbStatic);
	readAll(types.data(), nbDyn);
	readAll(geoms.data(), geoms.size());
	readAll(frictionOf.data(), nbDyn);
	readAll(staticPoses.data(), nbStatic);
	readAll(staticTypes.data(), nbStatic);
	readAll(staticGeoms.data(), staticGeoms.size());
	float prm[11];
	readAll(prm, 11);
	const float dt = prm[0];
	const PxVec3 gravity{prm[1], prm[2], prm[3]};
	const float contactDistance = prm[4], toleranceLength = prm[5], margin = prm[6], bounce = prm[7], frictionOffset = prm[8];
	const float correlation = prm[9], staticFriction = prm[10];
	const uint32_t nbPos = 4, nbVel = 1;
	const uint32_t nbTotal = nbDyn + nbStatic;

	std::vector<Shape> shapes(nbTotal);
	for(uint32_t i = 0; i < nbDyn; i++) shapes[i].set(types[i], &geoms[4 * size_t(i)]);
	for(uint32_t s = 0; s < nbStatic; s++) shapes[nbDyn + s].set(staticTypes[s], &staticGeoms[4 * size_t(s)]);
	CacheAllocator cacheAlloc;
	ConstraintAllocator alloc;
	std::map<std::pair<uint32_t, uint32_t>, PairState> state;

	for(uint32_t frame = 0; frame < nbFrames; frame++)
	{
		cacheAlloc.arena.nextFrame();
		alloc.rows.nextFrame();
		alloc.friction.nextFrame();
		std::vector<PxTransform> poses(nbTotal);
		std::vector<float> bounds(6 * size_t(nbTotal));
		for(uint32_t i = 0; i < nbTotal; i++)
		{
			poses[i] = i < nbDyn ? rigid[i].body2World : staticPoses[i - nbDyn];
			const float* g = i < nbDyn ? &geoms[4 * size_t(i)] : &staticGeoms[4 * size_t(i - nbDyn)];
			shapeBounds(i < nbDyn ? types[i] : staticTypes[i - nbDyn], g, poses[i], margin, &bounds[6 * size_t(i)]);
		}
		// overlapping pairs in (id0, id1) order; a pair keeps its state while it overlaps
		std::vector<std::pair<uint32_t, uint32_t>> pairs;
		for(uint32_t i = 0; i < nbDyn; i++)
			for(uint32_t j = i + 1; j < nbTotal; j++)
				if(overlap(&bounds[6 * size_t(i)], &bounds[6 * size_t(j)])) pairs.push_back(std::make_pair(i, j));
		std::map<std::pair<uint32_t, uint32_t>, PairState> next;
		for(const auto& p : pairs)
		{
			auto it = state.find(p);
			next[p] = it != state.end() ? it->second : PairState();
		}
		state.swap(next);
		const uint32_t nbPairs = uint32_t(pairs.size());

		// contacts, with the pairs' caches
		std::vector<const PxGeometry*> g0(nbPairs), g1(nbPairs);
		std::vector<PxTransform> p0(nbPairs), p1(nbPairs);
		std::vector<PxCache> caches(nbPairs);
		for(uint32_t k = 0; k < nbPairs; k++)
		{
			g0[k] = &shapes[pairs[k].first].any;
			g1[k] = &shapes[pairs[k].second].any;
			p0[k] = poses[pairs[k].first];
			p1[k] = poses[pairs[k].second];
			caches[k] = state[pairs[k]].cache;
		}
		Recorder rec;
		rec.perPair.resize(nbPairs);
		if(nbPairs && !PxGenerateContacts(g0.data(), g1.data(), p0.data(), p1.data(), caches.data(), nbPairs, rec, contactDistance, 0.01f,
		                                  toleranceLength, cacheAlloc))
			return 3;
		for(uint32_t k = 0; k < nbPairs; k++)
		{
			PairState& ps = state[pairs[k]];
			ps.cache = caches[k];
			if(rec.perPair[k].empty()) { ps.friction = nullptr; ps.nbFriction = 0; }   // no contact: friction data dropped
		}

		// solver bodies: dynamics in one array, statics on their own
		std::vector<PxTGSSolverBodyVel> vel(nbDyn);
		std::vector<PxTGSSolverBodyTxInertia> txI(nbDyn);
		std::vector<PxTGSSolverBodyData> data(nbDyn);
		PxConstructSolverBodiesTGS(rigid.data(), vel.data(), txI.data(), data.data(), nbDyn, gravity, dt, false);
		std::vector<PxTGSSolverBodyVel> sVel(nbStatic);
		std::vector<PxTGSSolverBodyTxInertia> sTxI(nbStatic);
		std::vector<PxTGSSolverBodyData> sData(nbStatic);
		for(uint32_t s = 0; s < nbStatic; s++) PxConstructStaticSolverBodyTGS(staticPoses[s], sVel[s], sTxI[s], sData[s]);
		auto velOf = [&](uint32_t b) { return b < nbDyn ? &vel[b] : &sVel[b - nbDyn]; };

		// one constraint per pair with contacts; material as the snippet's recorder sets it
		std::vector<uint32_t> cons;
		for(uint32_t k = 0; k < nbPairs; k++)
			if(!rec.perPair[k].empty())
			{
				cons.push_back(k);
				const uint32_t a = pairs[k].first, b = pairs[k].second;
				const float mu = (frictionOf[a] + (b < nbDyn ? frictionOf[b] : staticFriction)) * 0.5f;
				for(PxContactPoint& c : rec.perPair[k])
				{
					c.staticFriction = mu;
					c.dynamicFriction = mu;
					c.restitution = 0.0f;
					c.maxImpulse = 3.4e38f;
				}
			}
		const uint32_t nc = uint32_t(cons.size());
		std::vector<PxSolverConstraintDesc> descs(nc ? nc : 1);
		memset(descs.data(), 0, descs.size() * sizeof(PxSolverConstraintDesc));
		for(uint32_t i = 0; i < nc; i++)
		{
			const uint32_t a = pairs[cons[i]].first, b = pairs[cons[i]].second;
			descs[i].tgsBodyA = velOf(a);
			descs[i].tgsBodyB = velOf(b);
			descs[i].bodyADataIndex = a;
			descs[i].bodyBDataIndex = b;
			descs[i].linkIndexA = descs[i].linkIndexB = 0xffff;
			descs[i].constraintLengthOver16 = 0;   // eCONTACT_CONSTRAINT
		}
		std::vector<PxConstraintBatchHeader> headers(nc ? nc : 1);
		std::vector<PxSolverConstraintDesc> ordered(nc ? nc : 1);
		const uint32_t nbHeaders = nc ? PxBatchConstraintsTGS(descs.data(), nc, vel.data(), nbDyn, headers.data(), ordered.data(), nullptr, 0) : 0;

		// contact descriptors in solve order, with each pair's friction data from the last frame
		std::vector<uint32_t> pairOfOrdered(nc);
		for(uint32_t i = 0; i < nc; i++)
			for(uint32_t j = 0; j < nc; j++)
				if(descs[j].tgsBodyA == ordered[i].tgsBodyA && descs[j].tgsBodyB == ordered[i].tgsBodyB) { pairOfOrdered[i] = cons[j]; break; }
		std::vector<PxTGSSolverContactDesc> cdesc(nc ? nc : 1);
		memset(cdesc.data(), 0, cdesc.size() * sizeof(PxTGSSolverContactDesc));
		for(uint32_t i = 0; i < nc; i++)
		{
			const uint32_t k = pairOfOrdered[i];
			const uint32_t a = pairs[k].first, b = pairs[k].second;
			const PairState& ps = state[pairs[k]];
			PxTGSSolverContactDesc& d = cdesc[i];
			d.invMassScales = PxConstraintInvMassScale{1.0f, 1.0f, 1.0f, 1.0f};
			d.desc = &ordered[i];
			d.body0 = velOf(a);
			d.body1 = velOf(b);
			d.body0TxI = a < nbDyn ? &txI[a] : &sTxI[a - nbDyn];
			d.body1TxI = b < nbDyn ? &txI[b] : &sTxI[b - nbDyn];
			d.bodyData0 = a < nbDyn ? &data[a] : &sData[a - nbDyn];
			d.bodyData1 = b < nbDyn ? &data[b] : &sData[b - nbDyn];
			d.bodyFrame0 = poses[a];
			d.bodyFrame1 = poses[b];
			d.bodyState0 = a < nbDyn ? eDYNAMIC_BODY : eSTATIC_BODY;
			d.bodyState1 = b < nbDyn ? eDYNAMIC_BODY : eSTATIC_BODY;
			d.contacts = rec.perPair[k].data();
			d.numContacts = uint32_t(rec.perPair[k].size());
			d.frictionPtr = ps.friction;
			d.frictionCount = uint8_t(ps.nbFriction);
			d.maxCCDSeparation = 3.4e38f;
			d.maxImpulse = 3.4e38f;
			d.offsetSlop = 0.0f;
		}
		const float stepDt = dt / float(nbPos);
		if(nc && !PxCreateContactConstraintsTGS(headers.data(), nbHeaders, cdesc.data(), alloc, 1.0f / stepDt, 1.0f / dt, bounce, frictionOffset,
		                                        correlation))
			return 4;
		for(uint32_t i = 0; i < nc; i++)
		{
			PairState& ps = state[pairs[pairOfOrdered[i]]];
			ps.friction = cdesc[i].frictionPtr;
			ps.nbFriction = cdesc[i].frictionCount;
		}
		PxSolveConstraintsTGS(headers.data(), nbHeaders, ordered.data(), vel.data(), txI.data(), nbDyn, nbPos, nbVel, stepDt, 1.0f / stepDt, 0,
		                      nullptr, nullptr, nullptr);
		std::vector<PxTransform> outPose(poses.begin(), poses.begin() + nbDyn);
		PxIntegrateSolverBodiesTGS(vel.data(), txI.data(), outPose.data(), nbDyn, dt);
		for(uint32_t i = 0; i < nbDyn; i++)
		{
			rigid[i].linearVelocity = vel[i].linearVelocity;
			rigid[i].angularVelocity = vel[i].angularVelocity;
			rigid[i].body2World = outPose[i];
		}
		fwrite(rigid.data(), sizeof(PxRigidBodyData), nbDyn, stdout);
		fwrite(&nc, 4, 1, stdout);
	}
	return 0;
}
