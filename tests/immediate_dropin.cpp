// One immediate-mode frame written against the reference's interface
// (physx::immediate: PxGenerateContacts, PxConstructSolverBodiesTGS,
// PxConstructStaticSolverBodyTGS, PxBatchConstraintsTGS,
// PxCreateContactConstraintsTGS, PxSolveConstraintsTGS,
// PxIntegrateSolverBodiesTGS), the way the reference's immediate-mode snippet
// drives it, linked against libgbpx_immediate.so.  Used by
// tests/test_immediate_dropin_gpu.py.
//
// stdin (binary): nbDyn, nbStatic, nbPairs (u32); PxRigidBodyData[nbDyn];
// dynamic types (i32) and geometry (4 floats) per body; static poses
// (PxTransform), types and geometry; pairs (u32 a, b; statics numbered after
// the dynamic bodies); per pair friction (f32); params: dt, gravity xyz,
// contactDistance, toleranceLength, bounceThreshold, frictionOffsetThreshold,
// correlationDistance (9 floats).
// stdout (binary): per dynamic body linear velocity, world angular velocity
// (6 floats) and pose (7 floats); then the number of constraints (u32).
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

struct NoCache : PxCacheAllocator
{
	uint8_t* allocateCacheData(const uint32_t) override { return nullptr; }
};

struct Allocator : PxConstraintAllocator
{
	std::vector<void*> blocks;
	uint8_t* reserveConstraintData(const uint32_t byteSize) override
	{
		void* p = nullptr;
		if(posix_memalign(&p, 16, byteSize ? byteSize : 16)) return nullptr;
		blocks.push_back(p);
		return static_cast<uint8_t*>(p);
	}
	uint8_t* reserveFrictionData(const uint32_t byteSize) override { return reserveConstraintData(byteSize); }
	~Allocator() override { for(void* p : blocks) free(p); }
};
} // namespace

int main()
{
	uint32_t hdr[3];
	readAll(hdr, 3);
	const uint32_t nbDyn = hdr[0], nbStatic = hdr[1], nbPairs = hdr[2];
	std::vector<PxRigidBodyData> rigid(nbDyn);
	readAll(rigid.data(), nbDyn);
	std::vector<int> types(nbDyn), staticTypes(nbStatic);
	std::vector<float> geoms(4 * size_t(nbDyn)), staticGeoms(4 * size_t(nbStatic));
	std::vector<PxTransform> staticPoses(nbStatic);
	readAll(types.data(), nbDyn);
	readAll(geoms.data(), geoms.size());
	readAll(staticPoses.data(), nbStatic);
	readAll(staticTypes.data(), nbStatic);
	readAll(staticGeoms.data(), staticGeoms.size());
	std::vector<uint32_t> pairs(2 * size_t(nbPairs));
	std::vector<float> friction(nbPairs);
	readAll(pairs.data(), pairs.size());
	readAll(friction.data(), nbPairs);
	float prm[9];
	readAll(prm, 9);
	const float dt = prm[0];
	const PxVec3 gravity{prm[1], prm[2], prm[3]};
	const float contactDistance = prm[4], toleranceLength = prm[5], bounce = prm[6], frictionOffset = prm[7], correlation = prm[8];
	const uint32_t nbPos = 4, nbVel = 1;

	// shapes and poses of every body (dynamics, then statics)
	const uint32_t nbTotal = nbDyn + nbStatic;
	std::vector<Shape> shapes(nbTotal);
	std::vector<PxTransform> poses(nbTotal);
	for(uint32_t i = 0; i < nbDyn; i++) { shapes[i].set(types[i], &geoms[4 * size_t(i)]); poses[i] = rigid[i].body2World; }
	for(uint32_t s = 0; s < nbStatic; s++) { shapes[nbDyn + s].set(staticTypes[s], &staticGeoms[4 * size_t(s)]); poses[nbDyn + s] = staticPoses[s]; }

	// contacts
	std::vector<const PxGeometry*> g0(nbPairs), g1(nbPairs);
	std::vector<PxTransform> p0(nbPairs), p1(nbPairs);
	std::vector<PxCache> caches(nbPairs);
	memset(caches.data(), 0, caches.size() * sizeof(PxCache));
	for(uint32_t k = 0; k < nbPairs; k++)
	{
		g0[k] = &shapes[pairs[2 * k]].any;
		g1[k] = &shapes[pairs[2 * k + 1]].any;
		p0[k] = poses[pairs[2 * k]];
		p1[k] = poses[pairs[2 * k + 1]];
	}
	Recorder rec;
	rec.perPair.resize(nbPairs);
	NoCache cacheAlloc;
	if(!PxGenerateContacts(g0.data(), g1.data(), p0.data(), p1.data(), caches.data(), nbPairs, rec, contactDistance, 0.01f, toleranceLength,
	                       cacheAlloc))
		return 3;

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

	// one constraint per pair with contacts, friction and restitution on the points
	std::vector<uint32_t> cons;
	for(uint32_t k = 0; k < nbPairs; k++)
		if(!rec.perPair[k].empty())
		{
			cons.push_back(k);
			for(PxContactPoint& c : rec.perPair[k])
			{
				c.staticFriction = friction[k];
				c.dynamicFriction = friction[k];
				c.restitution = 0.0f;
				c.maxImpulse = 3.4e38f;
			}
		}
	const uint32_t nc = uint32_t(cons.size());
	std::vector<PxSolverConstraintDesc> descs(nc);
	memset(descs.data(), 0, descs.size() * sizeof(PxSolverConstraintDesc));
	for(uint32_t i = 0; i < nc; i++)
	{
		const uint32_t a = pairs[2 * cons[i]], b = pairs[2 * cons[i] + 1];
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

	// contact descriptors in solve order
	std::vector<uint32_t> pairOfOrdered(nc);
	for(uint32_t i = 0; i < nc; i++)
	{
		const PxTGSSolverBodyVel* pa = ordered[i].tgsBodyA;
		for(uint32_t j = 0; j < nc; j++)
			if(descs[j].tgsBodyA == pa && descs[j].tgsBodyB == ordered[i].tgsBodyB) { pairOfOrdered[i] = cons[j]; break; }
	}
	std::vector<PxTGSSolverContactDesc> cdesc(nc ? nc : 1);
	memset(cdesc.data(), 0, cdesc.size() * sizeof(PxTGSSolverContactDesc));
	for(uint32_t i = 0; i < nc; i++)
	{
		const uint32_t k = pairOfOrdered[i];
		const uint32_t a = pairs[2 * k], b = pairs[2 * k + 1];
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
		d.maxCCDSeparation = 3.4e38f;
		d.maxImpulse = 3.4e38f;
		d.offsetSlop = 0.0f;
	}
	Allocator alloc;
	const float stepDt = dt / float(nbPos);
	if(nc && !PxCreateContactConstraintsTGS(headers.data(), nbHeaders, cdesc.data(), alloc, 1.0f / stepDt, 1.0f / dt, bounce, frictionOffset,
	                                        correlation))
		return 4;
	PxSolveConstraintsTGS(headers.data(), nbHeaders, ordered.data(), vel.data(), txI.data(), nbDyn, nbPos, nbVel, stepDt, 1.0f / stepDt, 0, nullptr,
	                      nullptr, nullptr);
	std::vector<PxTransform> outPose(poses.begin(), poses.begin() + nbDyn);
	PxIntegrateSolverBodiesTGS(vel.data(), txI.data(), outPose.data(), nbDyn, dt);
	for(uint32_t i = 0; i < nbDyn; i++)
	{
		const float o[13] = {vel[i].linearVelocity.x, vel[i].linearVelocity.y, vel[i].linearVelocity.z, vel[i].angularVelocity.x,
		                     vel[i].angularVelocity.y, vel[i].angularVelocity.z, outPose[i].q.x, outPose[i].q.y, outPose[i].q.z,
		                     outPose[i].q.w, outPose[i].p.x, outPose[i].p.y, outPose[i].p.z};
		fwrite(o, 4, 13, stdout);
	}
	fwrite(&nc, 4, 1, stdout);
	return 0;
}
