// C harness over the reference PhysX immediate-mode API, compiled together with
// the reference's own sources by oracle/ref/Makefile into oracle/_ref/libpxref.so.
//
// Test infrastructure only: Python loads it with ctypes to produce golden
// fixtures and to pin the CPU restatement in oracle/port.  Every entry point
// is a thin adapter: plain arrays in, the reference function called exactly as
// its canonical caller (the immediate-mode snippet) calls it, plain arrays out.
//
// Layout conventions shared with the rest of the repository:
//   pose    = 7 floats  (qx, qy, qz, qw, px, py, pz)          -- PxTransform
//   geom    = type (PxGeometryType: 0 sphere, 1 plane, 2 capsule, 3 box, 4 convex core
//             with its PxConvexCore::Type in bits 8..15) +
//             4 floats (sphere: r; capsule: r, halfHeight; box: hx, hy, hz;
//             convex core: its core floats, margin in the fourth)
//   contact = 8 floats  (nx, ny, nz, separation, px, py, pz, 0)
#include "PxImmediateMode.h"
#include "PxBroadPhase.h"
#include "foundation/PxFoundation.h"
#include "foundation/PxPhysicsVersion.h"
#include "foundation/PxAllocatorCallback.h"
#include "foundation/PxErrorCallback.h"
#include "geometry/PxSphereGeometry.h"
#include "geometry/PxPlaneGeometry.h"
#include "geometry/PxCapsuleGeometry.h"
#include "geometry/PxBoxGeometry.h"
#include "geometry/PxConvexCoreGeometry.h"
#include "geomutils/PxContactPoint.h"
#include "collision/PxCollisionDefs.h"
#include "solver/PxSolverDefs.h"
#include "foundation/PxVecMath.h"

#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <vector>
#include <map>
#include <utility>
#include <algorithm>
#include <cmath>

using namespace physx;
using namespace physx::immediate;

#define HX extern "C" __attribute__((visibility("default")))

namespace
{
struct HAlloc : PxAllocatorCallback
{
	void* allocate(size_t size, const char*, const char*, int) override
	{
		void* p = nullptr;
		if(posix_memalign(&p, 16, size ? size : 16)) return nullptr;
		return p;
	}
	void deallocate(void* ptr) override { free(ptr); }
};
struct HErr : PxErrorCallback
{
	void reportError(PxErrorCode::Enum code, const char* message, const char* file, int line) override
	{
		fprintf(stderr, "[pxref] error %d: %s (%s:%d)\n", int(code), message, file, line);
	}
};
HAlloc gAlloc;
HErr gErr;
PxFoundation* gFoundation = nullptr;

void ensureFoundation()
{
	if(!gFoundation)
		gFoundation = PxCreateFoundation(PX_PHYSICS_VERSION, gAlloc, gErr);
}

// Bump arena with 16-byte alignment; reset wholesale.
struct Arena
{
	std::vector<PxU8*> blocks;
	PxU8* cur = nullptr;
	size_t used = 0, cap = 0;
	PxU8* alloc(size_t n)
	{
		n = (n + 15) & ~size_t(15);
		if(!cur || used + n > cap)
		{
			size_t sz = n > (1u << 20) ? n : (1u << 20);
			void* p = nullptr;
			if(posix_memalign(&p, 16, sz)) return nullptr;
			memset(p, 0, sz);
			blocks.push_back(static_cast<PxU8*>(p));
			cur = static_cast<PxU8*>(p);
			used = 0;
			cap = sz;
		}
		PxU8* r = cur + used;
		used += n;
		return r;
	}
	void reset()
	{
		for(PxU8* b : blocks) free(b);
		blocks.clear();
		cur = nullptr;
		used = cap = 0;
	}
	~Arena() { reset(); }
};

// Cache memory lives two frames, as the PxCacheAllocator contract asks.
struct FrameCacheAllocator : PxCacheAllocator
{
	Arena arenas[2];
	int frame = 0;
	PxU8* allocateCacheData(const PxU32 byteSize) override { return arenas[frame & 1].alloc(byteSize); }
	void nextFrame() { frame++; arenas[frame & 1].reset(); }
	void resetAll() { arenas[0].reset(); arenas[1].reset(); }
};

// Constraint rows live until the solve ends; friction data lives two frames.
struct FrameConstraintAllocator : PxConstraintAllocator
{
	Arena rows;
	Arena friction[2];
	int frame = 0;
	PxU8* reserveConstraintData(const PxU32 byteSize) override { return rows.alloc(byteSize); }
	PxU8* reserveFrictionData(const PxU32 byteSize) override { return friction[frame & 1].alloc(byteSize); }
	void nextFrame() { rows.reset(); frame++; friction[frame & 1].reset(); }
};

struct GeomHolder
{
	PxSphereGeometry sphere;
	PxPlaneGeometry plane;
	PxCapsuleGeometry capsule;
	PxBoxGeometry box;
	PxConvexCoreGeometry convex;
	const PxGeometry* set(int type, const float* p)
	{
		switch(type & 0xff)
		{
		case 0: sphere = PxSphereGeometry(p[0]); return &sphere;
		case 1: plane = PxPlaneGeometry(); return &plane;
		case 2: capsule = PxCapsuleGeometry(p[0], p[1]); return &capsule;
		case 3: box = PxBoxGeometry(p[0], p[1], p[2]); return &box;
		case 4:   // convex core: PxConvexCore::Type in bits 8..15, core floats, margin in p[3]
			switch((type >> 8) & 0xff)
			{
			case 0: convex = PxConvexCoreGeometry(PxConvexCore::Point(), p[3]); return &convex;
			case 1: convex = PxConvexCoreGeometry(PxConvexCore::Segment(p[0]), p[3]); return &convex;
			case 2: convex = PxConvexCoreGeometry(PxConvexCore::Box(p[0], p[1], p[2]), p[3]); return &convex;
			case 3: convex = PxConvexCoreGeometry(PxConvexCore::Ellipsoid(p[0], p[1], p[2]), p[3]); return &convex;
			case 4: convex = PxConvexCoreGeometry(PxConvexCore::Cylinder(p[0], p[1]), p[3]); return &convex;
			case 5: convex = PxConvexCoreGeometry(PxConvexCore::Cone(p[0], p[1]), p[3]); return &convex;
			default: return nullptr;
			}
		default: return nullptr;
		}
	}
};

PxTransform loadPose(const float* p)
{
	return PxTransform(PxVec3(p[4], p[5], p[6]), PxQuat(p[0], p[1], p[2], p[3]));
}

void storePose(float* o, const PxTransform& t)
{
	o[0] = t.q.x; o[1] = t.q.y; o[2] = t.q.z; o[3] = t.q.w;
	o[4] = t.p.x; o[5] = t.p.y; o[6] = t.p.z;
}

struct BufferRecorder : PxContactRecorder
{
	float* out;
	PxU32* counts;
	PxU32 maxPerPair;
	bool recordContacts(const PxContactPoint* c, PxU32 n, PxU32 index) override
	{
		counts[index] = n;
		for(PxU32 i = 0; i < n && i < maxPerPair; i++)
		{
			float* o = out + (size_t(index) * maxPerPair + i) * 8;
			o[0] = c[i].normal.x; o[1] = c[i].normal.y; o[2] = c[i].normal.z;
			o[3] = c[i].separation;
			o[4] = c[i].point.x; o[5] = c[i].point.y; o[6] = c[i].point.z;
			o[7] = 0.0f;
		}
		return true;
	}
};
} // namespace

//////////////////////////////////////////////////////////////////////////////
// Sizes of the public structures (checked against the GB300 build's mirrors).
HX int pxref_sizeof(int which)
{
	switch(which)
	{
	case 0: return int(sizeof(PxRigidBodyData));
	case 1: return int(sizeof(PxTGSSolverBodyVel));
	case 2: return int(sizeof(PxTGSSolverBodyTxInertia));
	case 3: return int(sizeof(PxTGSSolverBodyData));
	case 4: return int(sizeof(PxSolverConstraintDesc));
	case 5: return int(sizeof(PxConstraintBatchHeader));
	case 6: return int(sizeof(PxTGSSolverContactDesc));
	case 7: return int(sizeof(PxContactPoint));
	case 8: return int(sizeof(PxCache));
	case 9: return int(sizeof(PxBounds3));
	case 10: return int(sizeof(PxBroadPhasePair));
	case 11: return int(sizeof(PxTransform));
	case 12: return int(sizeof(Px1DConstraint));
	case 13: return int(sizeof(PxTGSSolverConstraintPrepDesc));
	default: return -1;
	}
}

//////////////////////////////////////////////////////////////////////////////
// Broadphase: PxCreateBroadPhase(eABP) + update/fetchResults.
HX void* pxref_bp_create_typed(int type, int discardStaticVsKinematic, int discardKinematicVsKinematic)
{
	ensureFoundation();
	PxBroadPhaseDesc desc(type == 1 ? PxBroadPhaseType::ePABP : PxBroadPhaseType::eABP);
	desc.mDiscardStaticVsKinematic = discardStaticVsKinematic != 0;
	desc.mDiscardKinematicVsKinematic = discardKinematicVsKinematic != 0;
	return PxCreateBroadPhase(desc);
}

HX void* pxref_bp_create(int discardStaticVsKinematic, int discardKinematicVsKinematic)
{
	ensureFoundation();
	PxBroadPhaseDesc desc(PxBroadPhaseType::eABP);
	desc.mDiscardStaticVsKinematic = discardStaticVsKinematic != 0;
	desc.mDiscardKinematicVsKinematic = discardKinematicVsKinematic != 0;
	return PxCreateBroadPhase(desc);
}

HX void pxref_bp_release(void* bp)
{
	if(bp) static_cast<PxBroadPhase*>(bp)->release();
}

HX PxU32 pxref_bp_filter_group(int kind, PxU32 id)
{
	ensureFoundation();
	if(kind == 0) return PxGetBroadPhaseStaticFilterGroup();
	if(kind == 1) return PxGetBroadPhaseKinematicFilterGroup(id);
	return PxGetBroadPhaseDynamicFilterGroup(id);
}

// bounds: 6 floats per object (minx miny minz maxx maxy maxz), capacity+1 entries
// (the reference may read 4 bytes past the last one).
HX int pxref_bp_update(void* bpv, const PxU32* created, PxU32 nbCreated, const PxU32* updated, PxU32 nbUpdated,
	const PxU32* removed, PxU32 nbRemoved, const float* bounds, const PxU32* groups, const float* distances, PxU32 capacity,
	PxU32* outCreated, PxU32 maxCreated, PxU32* nbOutCreated, PxU32* outLost, PxU32 maxLost, PxU32* nbOutLost)
{
	PxBroadPhase* bp = static_cast<PxBroadPhase*>(bpv);
	const PxBroadPhaseUpdateData data(created, nbCreated, updated, nbUpdated, removed, nbRemoved,
		reinterpret_cast<const PxBounds3*>(bounds), groups, distances, capacity);
	PxBroadPhaseResults results;
	bp->update(results, data);
	*nbOutCreated = results.mNbCreatedPairs;
	*nbOutLost = results.mNbDeletedPairs;
	for(PxU32 i = 0; i < results.mNbCreatedPairs && i < maxCreated; i++)
	{
		outCreated[2 * i] = results.mCreatedPairs[i].mID0;
		outCreated[2 * i + 1] = results.mCreatedPairs[i].mID1;
	}
	for(PxU32 i = 0; i < results.mNbDeletedPairs && i < maxLost; i++)
	{
		outLost[2 * i] = results.mDeletedPairs[i].mID0;
		outLost[2 * i + 1] = results.mDeletedPairs[i].mID1;
	}
	return (results.mNbCreatedPairs <= maxCreated && results.mNbDeletedPairs <= maxLost) ? 0 : 1;
}

//////////////////////////////////////////////////////////////////////////////
// Narrowphase: PxGenerateContacts, one pair per call as the snippet does, with
// a persistent PxCache per pair slot.
namespace
{
struct NpContext
{
	std::vector<PxCache> caches;
	FrameCacheAllocator alloc;
};
}

HX void* pxref_np_create(PxU32 nbPairs)
{
	ensureFoundation();
	NpContext* c = new NpContext;
	c->caches.resize(nbPairs);
	return c;
}

HX void pxref_np_release(void* c) { delete static_cast<NpContext*>(c); }

HX void pxref_np_reset(void* cv)
{
	NpContext* c = static_cast<NpContext*>(cv);
	for(PxCache& k : c->caches) k = PxCache();
	c->alloc.resetAll();
}

HX int pxref_np_run(void* cv, const int* type0, const float* geom0, const int* type1, const float* geom1,
	const float* pose0, const float* pose1, PxU32 nbPairs, float contactDistance, float meshContactMargin,
	float toleranceLength, int freshCaches, float* outContacts, PxU32 maxPerPair, PxU32* outCounts)
{
	NpContext* c = static_cast<NpContext*>(cv);
	if(nbPairs > c->caches.size()) c->caches.resize(nbPairs);
	c->alloc.nextFrame();
	BufferRecorder rec;
	rec.out = outContacts;
	rec.counts = outCounts;
	rec.maxPerPair = maxPerPair;
	int overflow = 0;
	for(PxU32 i = 0; i < nbPairs; i++)
	{
		outCounts[i] = 0;
		GeomHolder h0, h1;
		const PxGeometry* g0 = h0.set(type0[i], geom0 + 4 * i);
		const PxGeometry* g1 = h1.set(type1[i], geom1 + 4 * i);
		if(!g0 || !g1) return -1;
		const PxTransform t0 = loadPose(pose0 + 7 * i);
		const PxTransform t1 = loadPose(pose1 + 7 * i);
		if(freshCaches) c->caches[i] = PxCache();
		// The recorder indexes by the pair index passed here: rebase to slot i.
		struct Rebase : PxContactRecorder
		{
			BufferRecorder* r; PxU32 slot;
			bool recordContacts(const PxContactPoint* p, PxU32 n, PxU32) override { return r->recordContacts(p, n, slot); }
		} rb;
		rb.r = &rec;
		rb.slot = i;
		PxGenerateContacts(&g0, &g1, &t0, &t1, &c->caches[i], 1, rb, contactDistance, meshContactMargin, toleranceLength, c->alloc);
		if(outCounts[i] > maxPerPair) overflow = 1;
	}
	return overflow;
}

//////////////////////////////////////////////////////////////////////////////
// TGS bodies: PxConstructSolverBodiesTGS / PxConstructStaticSolverBodyTGS.
// rigid: nb x 96-byte PxRigidBodyData; outputs raw 64/64/48-byte records.
HX void pxref_construct_bodies_tgs(const void* rigid, PxU32 nb, const float* gravity, float dt,
	void* outVel, void* outTxI, void* outData)
{
	ensureFoundation();
	PxConstructSolverBodiesTGS(static_cast<const PxRigidBodyData*>(rigid), static_cast<PxTGSSolverBodyVel*>(outVel),
		static_cast<PxTGSSolverBodyTxInertia*>(outTxI), static_cast<PxTGSSolverBodyData*>(outData), nb,
		PxVec3(gravity[0], gravity[1], gravity[2]), dt, false);
}

HX void pxref_construct_static_body_tgs(const float* pose, void* outVel, void* outTxI, void* outData)
{
	ensureFoundation();
	PxConstructStaticSolverBodyTGS(loadPose(pose), *static_cast<PxTGSSolverBodyVel*>(outVel),
		*static_cast<PxTGSSolverBodyTxInertia*>(outTxI), *static_cast<PxTGSSolverBodyData*>(outData));
}

// Batching: constraint i joins body pairA[i], pairB[i]; indices >= nbDyn are
// static/kinematic (placed after the dynamic bodies in one array, as the
// snippet does).  Outputs headers (start, stride) and the order of the
// original constraint indices.
HX PxU32 pxref_batch_constraints_tgs(const PxU32* bodyA, const PxU32* bodyB, PxU32 nbConstraints, PxU32 nbDyn, PxU32 nbStatic,
	PxU32* outHeaderStart, PxU32* outHeaderStride, PxU32* outOrder)
{
	ensureFoundation();
	std::vector<PxTGSSolverBodyVel> bodies(nbDyn + nbStatic);
	memset(bodies.data(), 0, sizeof(PxTGSSolverBodyVel) * bodies.size());
	std::vector<PxSolverConstraintDesc> descs(nbConstraints), ordered(nbConstraints);
	std::vector<PxU32> ids(nbConstraints);
	for(PxU32 i = 0; i < nbConstraints; i++)
	{
		PxSolverConstraintDesc& d = descs[i];
		memset(&d, 0, sizeof(d));
		d.tgsBodyA = &bodies[bodyA[i]];
		d.tgsBodyB = &bodies[bodyB[i]];
		d.bodyADataIndex = bodyA[i];
		d.bodyBDataIndex = bodyB[i];
		d.linkIndexA = PxSolverConstraintDesc::RIGID_BODY;
		d.linkIndexB = PxSolverConstraintDesc::RIGID_BODY;
		ids[i] = i;
		d.constraint = reinterpret_cast<PxU8*>(&ids[i]);
		d.constraintType = PxSolverConstraintDesc::eCONTACT_CONSTRAINT;
	}
	std::vector<PxConstraintBatchHeader> headers(nbConstraints ? nbConstraints : 1);
	const PxU32 nbHeaders = PxBatchConstraintsTGS(descs.data(), nbConstraints, bodies.data(), nbDyn, headers.data(), ordered.data());
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		outHeaderStart[h] = headers[h].startIndex;
		outHeaderStride[h] = headers[h].stride;
	}
	for(PxU32 i = 0; i < nbConstraints; i++)
		outOrder[i] = *reinterpret_cast<const PxU32*>(ordered[i].constraint);
	return nbHeaders;
}

//////////////////////////////////////////////////////////////////////////////
// One TGS solve from given contacts, in the order the reference batches them:
// construct bodies, batch, create contact constraints, solve, integrate.
//
// rigid       nbDyn x PxRigidBodyData (96 B)
// staticPose  nbStatic x 7 floats
// pairA/B     body indices (>= nbDyn: static nbDyn+s)
// contactStart/contactCount per constraint into contacts (8 floats each)
// friction    per-constraint static/dynamic friction and restitution (3 floats)
// out*        velocities after solve (lin, ang: 6 floats per dynamic body, the
//             angular one in world space after PxIntegrateSolverBodiesTGS),
//             poses after integration (7 floats per dynamic body),
//             headers and order as pxref_batch_constraints_tgs.
// frictionPtr / frictionCount (per constraint, may be null): the friction data
// each constraint left last frame, replaced by what it leaves this frame (in
// alloc's friction memory, which lives two frames), as the snippet's persistent
// pairs keep it.
static PxU32 tgsFrameRef(const void* rigid, PxU32 nbDyn, const float* staticPose, PxU32 nbStatic,
	const PxU32* pairA, const PxU32* pairB, PxU32 nbConstraints, const PxU32* contactStart, const PxU32* contactCount,
	const float* contacts, const float* material, const float* gravity, float dt, PxU32 nbPos, PxU32 nbVel,
	float bounceThreshold, float frictionOffsetThreshold, float correlationDistance,
	float* outVel, float* outPose, PxU32* outHeaderStart, PxU32* outHeaderStride, PxU32* outOrder,
	void* outBodyVelRaw, void* outTxIRaw, FrameConstraintAllocator& alloc, PxU8** frictionPtr, PxU32* frictionCount)
{
	const PxU32 nbTotal = nbDyn + nbStatic;
	std::vector<PxTGSSolverBodyVel> bodies(nbTotal);
	std::vector<PxTGSSolverBodyTxInertia> txI(nbTotal);
	std::vector<PxTGSSolverBodyData> bodyData(nbTotal);
	std::vector<PxTransform> poses(nbTotal);
	const PxRigidBodyData* rb = static_cast<const PxRigidBodyData*>(rigid);
	const PxVec3 g(gravity[0], gravity[1], gravity[2]);
	for(PxU32 a = 0; a < nbDyn; a++)
	{
		PxConstructSolverBodiesTGS(&rb[a], &bodies[a], &txI[a], &bodyData[a], 1, g, dt, false);
		poses[a] = rb[a].body2World;
	}
	for(PxU32 s = 0; s < nbStatic; s++)
	{
		poses[nbDyn + s] = loadPose(staticPose + 7 * s);
		PxConstructStaticSolverBodyTGS(poses[nbDyn + s], bodies[nbDyn + s], txI[nbDyn + s], bodyData[nbDyn + s]);
	}

	// Contact points with the material fields the snippet's recorder fills in.
	PxU32 nbContactsTotal = 0;
	for(PxU32 i = 0; i < nbConstraints; i++)
		nbContactsTotal = PxMax(nbContactsTotal, contactStart[i] + contactCount[i]);
	std::vector<PxContactPoint> points(nbContactsTotal ? nbContactsTotal : 1);
	for(PxU32 i = 0; i < nbConstraints; i++)
	{
		for(PxU32 c = 0; c < contactCount[i]; c++)
		{
			const float* s = contacts + 8 * (contactStart[i] + c);
			PxContactPoint& p = points[contactStart[i] + c];
			memset(&p, 0, sizeof(p));
			p.normal = PxVec3(s[0], s[1], s[2]);
			p.separation = s[3];
			p.point = PxVec3(s[4], s[5], s[6]);
			p.maxImpulse = PX_MAX_F32;
			p.targetVel = PxVec3(0.0f);
			p.staticFriction = material[3 * i + 0];
			p.dynamicFriction = material[3 * i + 1];
			p.restitution = material[3 * i + 2];
			p.damping = 0.0f;
			p.materialFlags = 0;
		}
	}
	std::vector<PxReal> forces(nbContactsTotal ? nbContactsTotal : 1, 0.0f);

	std::vector<PxSolverConstraintDesc> descs(nbConstraints), ordered(nbConstraints);
	std::vector<PxU32> ids(nbConstraints);
	for(PxU32 i = 0; i < nbConstraints; i++)
	{
		PxSolverConstraintDesc& d = descs[i];
		memset(&d, 0, sizeof(d));
		d.tgsBodyA = &bodies[pairA[i]];
		d.tgsBodyB = &bodies[pairB[i]];
		d.bodyADataIndex = pairA[i];
		d.bodyBDataIndex = pairB[i];
		d.linkIndexA = PxSolverConstraintDesc::RIGID_BODY;
		d.linkIndexB = PxSolverConstraintDesc::RIGID_BODY;
		ids[i] = i;
		d.constraint = reinterpret_cast<PxU8*>(&ids[i]);
		d.constraintType = PxSolverConstraintDesc::eCONTACT_CONSTRAINT;
	}
	std::vector<PxConstraintBatchHeader> headers(nbConstraints ? nbConstraints : 1);
	const PxU32 nbHeaders = PxBatchConstraintsTGS(descs.data(), nbConstraints, bodies.data(), nbDyn, headers.data(), ordered.data());
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		outHeaderStart[h] = headers[h].startIndex;
		outHeaderStride[h] = headers[h].stride;
	}
	for(PxU32 i = 0; i < nbConstraints; i++)
		outOrder[i] = *reinterpret_cast<const PxU32*>(ordered[i].constraint);

	const PxReal invDt = 1.0f / dt;
	const PxReal stepDt = dt / PxReal(nbPos);
	const PxReal invStepDt = invDt * PxReal(nbPos);
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		PxConstraintBatchHeader& header = headers[h];
		PxTGSSolverContactDesc cd[4];
		for(PxU32 a = 0; a < header.stride; a++)
		{
			PxSolverConstraintDesc& desc = ordered[header.startIndex + a];
			const PxU32 ci = *reinterpret_cast<const PxU32*>(desc.constraint);
			PxTGSSolverContactDesc& c = cd[a];
			memset(&c, 0, sizeof(c));
			c.body0 = desc.tgsBodyA;
			c.body1 = desc.tgsBodyB;
			c.bodyData0 = &bodyData[desc.bodyADataIndex];
			c.bodyData1 = &bodyData[desc.bodyBDataIndex];
			c.body0TxI = &txI[desc.bodyADataIndex];
			c.body1TxI = &txI[desc.bodyBDataIndex];
			c.bodyFrame0 = poses[desc.bodyADataIndex];
			c.bodyFrame1 = poses[desc.bodyBDataIndex];
			c.contactForces = &forces[contactStart[ci]];
			c.contacts = &points[contactStart[ci]];
			c.numContacts = contactCount[ci];
			c.frictionPtr = frictionPtr ? frictionPtr[ci] : NULL;
			c.frictionCount = frictionCount ? PxU8(frictionCount[ci]) : 0;
			c.shapeInteraction = NULL;
			c.maxCCDSeparation = PX_MAX_F32;
			c.bodyState0 = desc.bodyADataIndex < nbDyn ? PxSolverConstraintPrepDescBase::eDYNAMIC_BODY : PxSolverConstraintPrepDescBase::eSTATIC_BODY;
			c.bodyState1 = desc.bodyBDataIndex < nbDyn ? PxSolverConstraintPrepDescBase::eDYNAMIC_BODY : PxSolverConstraintPrepDescBase::eSTATIC_BODY;
			c.desc = &desc;
			c.invMassScales.angular0 = c.invMassScales.angular1 = c.invMassScales.linear0 = c.invMassScales.linear1 = 1.0f;
		}
		PxCreateContactConstraintsTGS(&header, 1, cd, alloc, invStepDt, invDt, bounceThreshold, frictionOffsetThreshold, correlationDistance);
		for(PxU32 a = 0; frictionPtr && a < header.stride; a++)
		{
			const PxU32 ci = outOrder[header.startIndex + a];
			frictionPtr[ci] = cd[a].frictionPtr;
			frictionCount[ci] = cd[a].frictionCount;
		}
	}

	PxSolveConstraintsTGS(headers.data(), nbHeaders, ordered.data(), bodies.data(), txI.data(), nbDyn, nbPos, nbVel, stepDt, invStepDt);
	if(outBodyVelRaw) memcpy(outBodyVelRaw, bodies.data(), sizeof(PxTGSSolverBodyVel) * nbDyn);
	if(outTxIRaw) memcpy(outTxIRaw, txI.data(), sizeof(PxTGSSolverBodyTxInertia) * nbDyn);
	PxIntegrateSolverBodiesTGS(bodies.data(), txI.data(), poses.data(), nbDyn, dt);
	for(PxU32 a = 0; a < nbDyn; a++)
	{
		outVel[6 * a + 0] = bodies[a].linearVelocity.x;
		outVel[6 * a + 1] = bodies[a].linearVelocity.y;
		outVel[6 * a + 2] = bodies[a].linearVelocity.z;
		outVel[6 * a + 3] = bodies[a].angularVelocity.x;
		outVel[6 * a + 4] = bodies[a].angularVelocity.y;
		outVel[6 * a + 5] = bodies[a].angularVelocity.z;
		storePose(outPose + 7 * a, poses[a]);
	}
	return nbHeaders;
}

HX PxU32 pxref_tgs_solve(const void* rigid, PxU32 nbDyn, const float* staticPose, PxU32 nbStatic,
	const PxU32* pairA, const PxU32* pairB, PxU32 nbConstraints, const PxU32* contactStart, const PxU32* contactCount,
	const float* contacts, const float* material, const float* gravity, float dt, PxU32 nbPos, PxU32 nbVel,
	float bounceThreshold, float frictionOffsetThreshold, float correlationDistance,
	float* outVel, float* outPose, PxU32* outHeaderStart, PxU32* outHeaderStride, PxU32* outOrder,
	void* outBodyVelRaw, void* outTxIRaw)
{
	ensureFoundation();
	FrameConstraintAllocator alloc;
	return tgsFrameRef(rigid, nbDyn, staticPose, nbStatic, pairA, pairB, nbConstraints, contactStart, contactCount, contacts, material, gravity, dt,
		nbPos, nbVel, bounceThreshold, frictionOffsetThreshold, correlationDistance, outVel, outPose, outHeaderStart, outHeaderStride, outOrder,
		outBodyVelRaw, outTxIRaw, alloc, NULL, NULL);
}

//////////////////////////////////////////////////////////////////////////////
// One PGS solve from given contacts, as the immediate-mode snippet's PGS branch
// runs it (SnippetImmediateMode.cpp:749,761,961,1080-1099): PxConstructSolverBodies /
// PxConstructStaticSolverBody, PxBatchConstraints (batch != 0; else one header
// per constraint, typed as PxCreateContactConstraints types them), PxCreateContactConstraints
// per header, the solver bodies zeroed, PxSolveConstraints,
// PxIntegrateSolverBodies.  Inputs as pxref_tgs_solve.
// out*        velocities and poses of the dynamic bodies after integration
//             (PxSolverBodyData linear / angular velocity, body2World);
//             headers (start, stride, constraintType) and the constraint order;
//             outForces: per contact the normal impulse the last velocity
//             iteration wrote back (PxSolverContactDesc::contactForces).
HX PxU32 pxref_pgs_solve(const void* rigid, PxU32 nbDyn, const float* staticPose, PxU32 nbStatic,
	const PxU32* pairA, const PxU32* pairB, PxU32 nbConstraints, const PxU32* contactStart, const PxU32* contactCount,
	const float* contacts, const float* material, const float* gravity, float dt, PxU32 nbPos, PxU32 nbVel,
	float bounceThreshold, float frictionOffsetThreshold, float correlationDistance, int batch,
	float* outVel, float* outPose, PxU32* outHeaderStart, PxU32* outHeaderStride, PxU32* outHeaderType, PxU32* outOrder, float* outForces)
{
	ensureFoundation();
	FrameConstraintAllocator alloc;
	const PxU32 nbTotal = nbDyn + nbStatic;
	std::vector<PxSolverBody> bodies(nbTotal);
	std::vector<PxSolverBodyData> bodyData(nbTotal);
	const PxRigidBodyData* rb = static_cast<const PxRigidBodyData*>(rigid);
	const PxVec3 g(gravity[0], gravity[1], gravity[2]);
	for(PxU32 a = 0; a < nbDyn; a++)
		PxConstructSolverBodies(&rb[a], &bodyData[a], 1, g, dt, false);
	for(PxU32 s = 0; s < nbStatic; s++)
		PxConstructStaticSolverBody(loadPose(staticPose + 7 * s), bodyData[nbDyn + s]);

	PxU32 nbContactsTotal = 0;
	for(PxU32 i = 0; i < nbConstraints; i++)
		nbContactsTotal = PxMax(nbContactsTotal, contactStart[i] + contactCount[i]);
	std::vector<PxContactPoint> points(nbContactsTotal ? nbContactsTotal : 1);
	for(PxU32 i = 0; i < nbConstraints; i++)
	{
		for(PxU32 c = 0; c < contactCount[i]; c++)
		{
			const float* s = contacts + 8 * (contactStart[i] + c);
			PxContactPoint& p = points[contactStart[i] + c];
			memset(&p, 0, sizeof(p));
			p.normal = PxVec3(s[0], s[1], s[2]);
			p.separation = s[3];
			p.point = PxVec3(s[4], s[5], s[6]);
			p.maxImpulse = PX_MAX_F32;
			p.targetVel = PxVec3(0.0f);
			p.staticFriction = material[3 * i + 0];
			p.dynamicFriction = material[3 * i + 1];
			p.restitution = material[3 * i + 2];
			p.damping = 0.0f;
			p.materialFlags = 0;
		}
	}
	std::vector<PxReal> forces(nbContactsTotal ? nbContactsTotal : 1, 0.0f);

	std::vector<PxSolverConstraintDesc> descs(nbConstraints), ordered(nbConstraints);
	std::vector<PxU32> ids(nbConstraints);
	for(PxU32 i = 0; i < nbConstraints; i++)
	{
		PxSolverConstraintDesc& d = descs[i];
		memset(&d, 0, sizeof(d));
		d.bodyA = &bodies[pairA[i]];
		d.bodyB = &bodies[pairB[i]];
		d.bodyADataIndex = pairA[i];
		d.bodyBDataIndex = pairB[i];
		d.linkIndexA = PxSolverConstraintDesc::RIGID_BODY;
		d.linkIndexB = PxSolverConstraintDesc::RIGID_BODY;
		ids[i] = i;
		d.constraint = reinterpret_cast<PxU8*>(&ids[i]);
		d.constraintType = PxSolverConstraintDesc::eCONTACT_CONSTRAINT;
	}
	std::vector<PxConstraintBatchHeader> headers(nbConstraints ? nbConstraints : 1);
	PxU32 nbHeaders = 0;
	if(batch)
		nbHeaders = PxBatchConstraints(descs.data(), nbConstraints, bodies.data(), nbDyn, headers.data(), ordered.data());
	else
	{
		for(PxU32 i = 0; i < nbConstraints; i++)
		{
			headers[i].startIndex = i;
			headers[i].stride = 1;
			headers[i].constraintType = PxSolverConstraintDesc::eCONTACT_CONSTRAINT;
			ordered[i] = descs[i];
		}
		nbHeaders = nbConstraints;
	}
	for(PxU32 i = 0; i < nbConstraints; i++)
		outOrder[i] = *reinterpret_cast<const PxU32*>(ordered[i].constraint);

	const PxReal invDt = 1.0f / dt;
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		PxConstraintBatchHeader& header = headers[h];
		PxSolverContactDesc cd[4];
		for(PxU32 a = 0; a < header.stride; a++)
		{
			PxSolverConstraintDesc& desc = ordered[header.startIndex + a];
			const PxU32 ci = *reinterpret_cast<const PxU32*>(desc.constraint);
			PxSolverContactDesc& c = cd[a];
			memset(&c, 0, sizeof(c));
			c.body0 = desc.bodyA;
			c.body1 = desc.bodyB;
			c.data0 = &bodyData[desc.bodyADataIndex];
			c.data1 = &bodyData[desc.bodyBDataIndex];
			c.bodyFrame0 = c.data0->body2World;
			c.bodyFrame1 = c.data1->body2World;
			c.contactForces = &forces[contactStart[ci]];
			c.contacts = &points[contactStart[ci]];
			c.numContacts = contactCount[ci];
			c.frictionPtr = NULL;
			c.frictionCount = 0;
			c.shapeInteraction = NULL;
			c.maxCCDSeparation = PX_MAX_F32;
			c.bodyState0 = PxSolverConstraintPrepDescBase::eDYNAMIC_BODY;
			c.bodyState1 = desc.bodyBDataIndex < nbDyn ? PxSolverConstraintPrepDescBase::eDYNAMIC_BODY : PxSolverConstraintPrepDescBase::eSTATIC_BODY;
			c.desc = &desc;
			c.invMassScales.angular0 = c.invMassScales.angular1 = c.invMassScales.linear0 = c.invMassScales.linear1 = 1.0f;
		}
		PxCreateContactConstraints(&header, 1, cd, alloc, invDt, bounceThreshold, frictionOffsetThreshold, correlationDistance);
	}
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		outHeaderStart[h] = headers[h].startIndex;
		outHeaderStride[h] = headers[h].stride;
		outHeaderType[h] = headers[h].constraintType;
	}
	std::vector<PxVec3> motionLin(nbDyn ? nbDyn : 1), motionAng(nbDyn ? nbDyn : 1);
	PxMemZero(bodies.data(), bodies.size() * sizeof(PxSolverBody));
	PxSolveConstraints(headers.data(), nbHeaders, ordered.data(), bodies.data(), motionLin.data(), motionAng.data(), nbDyn, nbPos, nbVel);
	PxIntegrateSolverBodies(bodyData.data(), bodies.data(), motionLin.data(), motionAng.data(), nbDyn, dt);
	for(PxU32 a = 0; a < nbDyn; a++)
	{
		const PxSolverBodyData& d = bodyData[a];
		outVel[6 * a + 0] = d.linearVelocity.x;
		outVel[6 * a + 1] = d.linearVelocity.y;
		outVel[6 * a + 2] = d.linearVelocity.z;
		outVel[6 * a + 3] = d.angularVelocity.x;
		outVel[6 * a + 4] = d.angularVelocity.y;
		outVel[6 * a + 5] = d.angularVelocity.z;
		storePose(outPose + 7 * a, d.body2World);
	}
	if(outForces) memcpy(outForces, forces.data(), sizeof(float) * nbContactsTotal);
	return nbHeaders;
}

//////////////////////////////////////////////////////////////////////////////
// One TGS frame of joints, built as the immediate-mode snippet builds its
// joints (SnippetImmediateMode.cpp:838-1061) but with the caller's 1D rows in
// place of a joint shader: construct bodies, PxBatchConstraintsTGS over the
// joints, PxCreateJointConstraintsTGS per header, PxSolveConstraintsTGS,
// PxIntegrateSolverBodiesTGS.
//
// jointA/B          body indices (>= nbDyn: static nbDyn+s)
// rowStart/rowCount per joint into rows (Px1DConstraint, 80 B each; copied,
//                   the prep rewrites them)
// params            per joint 20 floats: invMassScales (linear0, angular0,
//                   linear1, angular1), cA2w, cB2w, body0WorldOffset,
//                   linBreakForce, angBreakForce, minResponseThreshold, flags
//                   (float holding 1 disablePreprocessing | 2 improvedSlerp |
//                   4 driveLimitsAreForces), 3 unused
// out*              velocities and poses as pxref_tgs_solve; headers with their
//                   constraint type (DY_SC_TYPE_*); per joint the write-back's
//                   linear and angular impulse (6 floats) and broken flag
// batchJoints       0: one header of stride 1 per joint in input order (the
//                   snippet without BATCH_CONTACTS), else PxBatchConstraintsTGS
namespace
{
struct JointWriteback   // Dy::ConstraintWriteback (DyConstraintWriteBack.h:42)
{
	PxVec3 linearImpulse;
	PxU32 broken;
	PxVec3 angularImpulse;
	PxReal residual;
};
}

HX PxU32 pxref_joint_frame(const void* rigid, PxU32 nbDyn, const float* staticPose, PxU32 nbStatic,
	const PxU32* jointA, const PxU32* jointB, PxU32 nbJoints, const PxU32* rowStart, const PxU32* rowCount, const void* rows,
	const float* params, const float* gravity, float dt, PxU32 nbPos, PxU32 nbVel, PxU32 batchJoints,
	float* outVel, float* outPose, PxU32* outHeaderStart, PxU32* outHeaderStride, PxU32* outHeaderType, PxU32* outOrder,
	float* outForce, PxU32* outBroken)
{
	ensureFoundation();
	const PxU32 nbTotal = nbDyn + nbStatic;
	std::vector<PxTGSSolverBodyVel> bodies(nbTotal);
	std::vector<PxTGSSolverBodyTxInertia> txI(nbTotal);
	std::vector<PxTGSSolverBodyData> bodyData(nbTotal);
	std::vector<PxTransform> poses(nbTotal);
	const PxRigidBodyData* rb = static_cast<const PxRigidBodyData*>(rigid);
	const PxVec3 g(gravity[0], gravity[1], gravity[2]);
	for(PxU32 a = 0; a < nbDyn; a++)
	{
		PxConstructSolverBodiesTGS(&rb[a], &bodies[a], &txI[a], &bodyData[a], 1, g, dt, false);
		poses[a] = rb[a].body2World;
	}
	for(PxU32 s = 0; s < nbStatic; s++)
	{
		poses[nbDyn + s] = loadPose(staticPose + 7 * s);
		PxConstructStaticSolverBodyTGS(poses[nbDyn + s], bodies[nbDyn + s], txI[nbDyn + s], bodyData[nbDyn + s]);
	}
	PxU32 nbRowsTotal = 0;
	for(PxU32 j = 0; j < nbJoints; j++) nbRowsTotal = PxMax(nbRowsTotal, rowStart[j] + rowCount[j]);
	std::vector<Px1DConstraint> rowCopy(nbRowsTotal ? nbRowsTotal : 1);
	if(nbRowsTotal) memcpy(rowCopy.data(), rows, sizeof(Px1DConstraint) * nbRowsTotal);
	std::vector<JointWriteback> writeback(nbJoints ? nbJoints : 1);
	memset(writeback.data(), 0, sizeof(JointWriteback) * writeback.size());

	std::vector<PxSolverConstraintDesc> descs(nbJoints), ordered(nbJoints);
	std::vector<PxU32> ids(nbJoints);
	for(PxU32 i = 0; i < nbJoints; i++)
	{
		PxSolverConstraintDesc& d = descs[i];
		memset(&d, 0, sizeof(d));
		d.tgsBodyA = &bodies[jointA[i]];
		d.tgsBodyB = &bodies[jointB[i]];
		d.bodyADataIndex = jointA[i];
		d.bodyBDataIndex = jointB[i];
		d.linkIndexA = PxSolverConstraintDesc::RIGID_BODY;
		d.linkIndexB = PxSolverConstraintDesc::RIGID_BODY;
		ids[i] = i;
		d.constraint = reinterpret_cast<PxU8*>(&ids[i]);
		d.constraintType = PxSolverConstraintDesc::eJOINT_CONSTRAINT;
	}
	std::vector<PxConstraintBatchHeader> headers(nbJoints ? nbJoints : 1);
	PxU32 nbHeaders = nbJoints;
	if(batchJoints)
		nbHeaders = PxBatchConstraintsTGS(descs.data(), nbJoints, bodies.data(), nbDyn, headers.data(), ordered.data());
	else
	{
		// the snippet's unbatched path: one header of stride 1 per joint, in input order
		for(PxU32 i = 0; i < nbJoints; i++)
		{
			headers[i].startIndex = i;
			headers[i].stride = 1;
			headers[i].constraintType = PxSolverConstraintDesc::eJOINT_CONSTRAINT;
			ordered[i] = descs[i];
		}
	}
	for(PxU32 i = 0; i < nbJoints; i++)
		outOrder[i] = *reinterpret_cast<const PxU32*>(ordered[i].constraint);

	const PxReal invDt = 1.0f / dt;
	const PxReal stepDt = dt / PxReal(nbPos);
	const PxReal invStepDt = invDt * PxReal(nbPos);
	FrameConstraintAllocator alloc;
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		PxConstraintBatchHeader& header = headers[h];
		PxTGSSolverConstraintPrepDesc jd[4];
		for(PxU32 a = 0; a < header.stride; a++)
		{
			PxSolverConstraintDesc& desc = ordered[header.startIndex + a];
			const PxU32 ji = *reinterpret_cast<const PxU32*>(desc.constraint);
			const float* pr = params + 20 * ji;
			PxTGSSolverConstraintPrepDesc& c = jd[a];
			memset(&c, 0, sizeof(c));
			c.body0 = desc.tgsBodyA;
			c.body1 = desc.tgsBodyB;
			c.bodyData0 = &bodyData[desc.bodyADataIndex];
			c.bodyData1 = &bodyData[desc.bodyBDataIndex];
			c.body0TxI = &txI[desc.bodyADataIndex];
			c.body1TxI = &txI[desc.bodyBDataIndex];
			c.bodyFrame0 = poses[desc.bodyADataIndex];
			c.bodyFrame1 = poses[desc.bodyBDataIndex];
			c.bodyState0 = desc.bodyADataIndex < nbDyn ? PxSolverConstraintPrepDescBase::eDYNAMIC_BODY : PxSolverConstraintPrepDescBase::eSTATIC_BODY;
			c.bodyState1 = desc.bodyBDataIndex < nbDyn ? PxSolverConstraintPrepDescBase::eDYNAMIC_BODY : PxSolverConstraintPrepDescBase::eSTATIC_BODY;
			c.desc = &desc;
			c.writeback = &writeback[ji];
			c.invMassScales = PxConstraintInvMassScale(pr[0], pr[1], pr[2], pr[3]);
			c.cA2w = PxVec3(pr[4], pr[5], pr[6]);
			c.cB2w = PxVec3(pr[7], pr[8], pr[9]);
			c.body0WorldOffset = PxVec3(pr[10], pr[11], pr[12]);
			c.linBreakForce = pr[13];
			c.angBreakForce = pr[14];
			c.minResponseThreshold = pr[15];
			const PxU32 fl = PxU32(pr[16]);
			c.disablePreprocessing = (fl & 1u) != 0;
			c.improvedSlerp = (fl & 2u) != 0;
			c.driveLimitsAreForces = (fl & 4u) != 0;
			c.rows = rowCopy.data() + rowStart[ji];
			c.numRows = rowCount[ji];
		}
		PxCreateJointConstraintsTGS(&header, 1, jd, alloc, stepDt, dt, invStepDt, invDt, 1.0f);
	}
	for(PxU32 h = 0; h < nbHeaders; h++)
	{
		outHeaderStart[h] = headers[h].startIndex;
		outHeaderStride[h] = headers[h].stride;
		outHeaderType[h] = headers[h].constraintType;
	}

	PxSolveConstraintsTGS(headers.data(), nbHeaders, ordered.data(), bodies.data(), txI.data(), nbDyn, nbPos, nbVel, stepDt, invStepDt);
	PxIntegrateSolverBodiesTGS(bodies.data(), txI.data(), poses.data(), nbDyn, dt);
	for(PxU32 a = 0; a < nbDyn; a++)
	{
		outVel[6 * a + 0] = bodies[a].linearVelocity.x;
		outVel[6 * a + 1] = bodies[a].linearVelocity.y;
		outVel[6 * a + 2] = bodies[a].linearVelocity.z;
		outVel[6 * a + 3] = bodies[a].angularVelocity.x;
		outVel[6 * a + 4] = bodies[a].angularVelocity.y;
		outVel[6 * a + 5] = bodies[a].angularVelocity.z;
		storePose(outPose + 7 * a, poses[a]);
	}
	for(PxU32 j = 0; j < nbJoints; j++)
	{
		const JointWriteback& w = writeback[j];
		outForce[6 * j + 0] = w.linearImpulse.x;
		outForce[6 * j + 1] = w.linearImpulse.y;
		outForce[6 * j + 2] = w.linearImpulse.z;
		outForce[6 * j + 3] = w.angularImpulse.x;
		outForce[6 * j + 4] = w.angularImpulse.y;
		outForce[6 * j + 5] = w.angularImpulse.z;
		outBroken[j] = (w.broken & 0x80000000u) ? 1u : 0u;
	}
	return nbHeaders;
}

//////////////////////////////////////////////////////////////////////////////
// One frame of the immediate-mode loop for many independent scenes, through
// the reference: bounds (shape AABB + margin, same arithmetic as the GB300
// build and the oracle) -> PxBroadPhase(eABP) with every object created (a
// fresh broadphase per frame) -> pairs sorted by (id0, id1) ->
// PxGenerateContacts (fresh caches) -> pxref_tgs_solve -> write-back.
namespace
{
void sceneShapeBounds(int type, const float* g, const float* pose7, float margin, float* out)
{
	const float qx = pose7[0], qy = pose7[1], qz = pose7[2], qw = pose7[3];
	float e[3];
	if(type == 0) { e[0] = e[1] = e[2] = g[0]; }
	else if(type == 2)
	{
		// QuatGetBasisVector0 (aos order)
		const float x2 = qx * 2.0f, w2 = qw * 2.0f;
		const float ax = (qw * w2 + qx * x2) - 1.0f, ay = qz * w2 + qy * x2, az = (-qy) * w2 + qz * x2;
		e[0] = fabsf(ax) * g[1] + g[0]; e[1] = fabsf(ay) * g[1] + g[0]; e[2] = fabsf(az) * g[1] + g[0];
	}
	else if(type == 3)
	{
		// QuatGetMat33V column form (PxVecMathSSE.h)
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
	for(int k = 0; k < 3; k++) { out[k] = (pose7[4 + k] - e[k]) - margin; out[3 + k] = (pose7[4 + k] + e[k]) + margin; }
}
}

// Persistent pair state across frames, as the snippet keeps it with
// WITH_PERSISTENCY (SnippetImmediateMode.cpp:47, 563-600, 657-676, 941-978):
// per overlapping pair its PxCache and the friction data its contact
// constraint left; a pair gets fresh state when the broadphase reports it and
// loses it when the pair stops overlapping; friction data is dropped for a
// pair whose contact generation found no contact.
namespace
{
struct PairStateRef
{
	PxCache cache;
	PxU8* frictions = NULL;
	PxU32 nbFrictions = 0;
};
struct PersistentRef
{
	std::vector<std::map<std::pair<PxU32, PxU32>, PairStateRef>> scenes;
	FrameCacheAllocator cacheAlloc;
	FrameConstraintAllocator constraintAlloc;
};

int sceneStepRef(PersistentRef* ps, PxU32 nbScenes, const PxU32* sceneBodyCount, const PxU32* sceneStaticCount, void* rigidIO, const int* types,
	const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
	const float* params, const PxU32* iterations);
}

HX void* pxref_persistent_create()
{
	ensureFoundation();
	return new PersistentRef;
}

HX void pxref_persistent_release(void* h) { delete static_cast<PersistentRef*>(h); }

// pxref_scene_step with persistent contact caches and friction data (state in h).
HX int pxref_scene_step_persistent(void* h, PxU32 nbScenes, const PxU32* sceneBodyCount, const PxU32* sceneStaticCount, void* rigidIO,
	const int* types, const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
	const float* params, const PxU32* iterations)
{
	return sceneStepRef(static_cast<PersistentRef*>(h), nbScenes, sceneBodyCount, sceneStaticCount, rigidIO, types, geoms, friction, staticPoses,
		staticTypes, staticGeoms, params, iterations);
}

HX int pxref_scene_step(PxU32 nbScenes, const PxU32* sceneBodyCount, const PxU32* sceneStaticCount, void* rigidIO, const int* types,
	const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
	const float* params, const PxU32* iterations)
{
	return sceneStepRef(NULL, nbScenes, sceneBodyCount, sceneStaticCount, rigidIO, types, geoms, friction, staticPoses, staticTypes, staticGeoms,
		params, iterations);
}

namespace
{
int sceneStepRef(PersistentRef* ps, PxU32 nbScenes, const PxU32* sceneBodyCount, const PxU32* sceneStaticCount, void* rigidIO, const int* types,
	const float* geoms, const float* friction, const float* staticPoses, const int* staticTypes, const float* staticGeoms,
	const float* params, const PxU32* iterations)
{
	ensureFoundation();
	if(ps)
	{
		if(ps->scenes.size() < nbScenes) ps->scenes.resize(nbScenes);
		ps->cacheAlloc.nextFrame();
		ps->constraintAlloc.nextFrame();
	}
	PxRigidBodyData* rigid = static_cast<PxRigidBodyData*>(rigidIO);
	const float dt = params[0];
	const float cDist = params[4], tolLen = params[5], margin = params[6];
	PxU32 b0 = 0, s0 = 0;
	for(PxU32 s = 0; s < nbScenes; s++)
	{
		const PxU32 n = sceneBodyCount[s], m = sceneStaticCount[s];
		std::vector<float> bounds(6 * size_t(n + m + 1), 0.0f), pose(7 * size_t(n + m)), geom(4 * size_t(n + m));
		std::vector<int> type(n + m);
		std::vector<PxU32> handles(n + m), groups(n + m);
		std::vector<float> dist(n + m, 0.0f);
		for(PxU32 i = 0; i < n + m; i++)
		{
			if(i < n)
			{
				const PxRigidBodyData& r = rigid[b0 + i];
				const float p7[7] = {r.body2World.q.x, r.body2World.q.y, r.body2World.q.z, r.body2World.q.w, r.body2World.p.x, r.body2World.p.y, r.body2World.p.z};
				memcpy(&pose[7 * i], p7, 28);
				type[i] = types[b0 + i];
				memcpy(&geom[4 * i], geoms + 4 * size_t(b0 + i), 16);
				groups[i] = PxGetBroadPhaseDynamicFilterGroup(i);
			}
			else
			{
				memcpy(&pose[7 * i], staticPoses + 7 * size_t(s0 + i - n), 28);
				type[i] = staticTypes[s0 + i - n];
				memcpy(&geom[4 * i], staticGeoms + 4 * size_t(s0 + i - n), 16);
				groups[i] = PxGetBroadPhaseStaticFilterGroup();
			}
			sceneShapeBounds(type[i], &geom[4 * i], &pose[7 * i], margin, &bounds[6 * i]);
			handles[i] = i;
		}
		PxBroadPhaseDesc bpDesc(PxBroadPhaseType::eABP);
		PxBroadPhase* bp = PxCreateBroadPhase(bpDesc);
		const PxBroadPhaseUpdateData ud(handles.data(), n + m, NULL, 0, NULL, 0, reinterpret_cast<const PxBounds3*>(bounds.data()), groups.data(),
			dist.data(), n + m);
		PxBroadPhaseResults res;
		bp->update(res, ud);
		std::vector<std::pair<PxU32, PxU32>> pairs;
		for(PxU32 k = 0; k < res.mNbCreatedPairs; k++)
		{
			PxU32 a = res.mCreatedPairs[k].mID0, b = res.mCreatedPairs[k].mID1;
			if(a > b) std::swap(a, b);
			pairs.push_back(std::make_pair(a, b));
		}
		bp->release();
		std::sort(pairs.begin(), pairs.end());
		const size_t np = pairs.size();
		std::vector<int> t0(np), t1(np);
		std::vector<float> g0(4 * np), g1(4 * np), p0(7 * np), p1(7 * np);
		for(size_t k = 0; k < np; k++)
		{
			const PxU32 a = pairs[k].first, b = pairs[k].second;
			t0[k] = type[a]; t1[k] = type[b];
			memcpy(&g0[4 * k], &geom[4 * a], 16); memcpy(&g1[4 * k], &geom[4 * b], 16);
			memcpy(&p0[7 * k], &pose[7 * a], 28); memcpy(&p1[7 * k], &pose[7 * b], 28);
		}
		std::vector<float> cts(np * 8 * 8 + 8);
		std::vector<PxU32> cnt(np + 1);
		std::vector<PairStateRef*> state(np, NULL);
		if(ps)
		{
			// pairs that stopped overlapping lose their state; new ones start fresh
			std::map<std::pair<PxU32, PxU32>, PairStateRef> next;
			std::map<std::pair<PxU32, PxU32>, PairStateRef>& cur = ps->scenes[s];
			for(size_t k = 0; k < np; k++)
			{
				auto it = cur.find(pairs[k]);
				next[pairs[k]] = it != cur.end() ? it->second : PairStateRef();
			}
			cur.swap(next);
			for(size_t k = 0; k < np; k++) state[k] = &cur[pairs[k]];
			BufferRecorder rec;
			rec.out = cts.data();
			rec.counts = cnt.data();
			rec.maxPerPair = 8;
			for(size_t k = 0; k < np; k++)
			{
				cnt[k] = 0;
				GeomHolder h0, h1;
				const PxGeometry* gg0 = h0.set(t0[k], &g0[4 * k]);
				const PxGeometry* gg1 = h1.set(t1[k], &g1[4 * k]);
				const PxTransform tr0 = loadPose(&p0[7 * k]), tr1 = loadPose(&p1[7 * k]);
				struct Rebase : PxContactRecorder
				{
					BufferRecorder* r; PxU32 slot;
					bool recordContacts(const PxContactPoint* p, PxU32 nn, PxU32) override { return r->recordContacts(p, nn, slot); }
				} rb;
				rb.r = &rec;
				rb.slot = PxU32(k);
				PxGenerateContacts(&gg0, &gg1, &tr0, &tr1, &state[k]->cache, 1, rb, cDist, 0.01f, tolLen, ps->cacheAlloc);
				if(!cnt[k]) { state[k]->frictions = NULL; state[k]->nbFrictions = 0; }
			}
		}
		else
		{
			void* np_ = pxref_np_create(PxU32(np));
			if(np) pxref_np_run(np_, t0.data(), g0.data(), t1.data(), g1.data(), p0.data(), p1.data(), PxU32(np), cDist, 0.01f, tolLen, 1, cts.data(), 8, cnt.data());
			pxref_np_release(np_);
		}
		std::vector<PxU32> ca, cb, cs, cc, fcount;
		std::vector<float> packed, mat;
		std::vector<PxU8*> fptr;
		std::vector<PairStateRef*> cstate;
		for(size_t k = 0; k < np; k++)
		{
			if(!cnt[k]) continue;
			if(ps)
			{
				cstate.push_back(state[k]);
				fptr.push_back(state[k]->frictions);
				fcount.push_back(state[k]->nbFrictions);
			}
			ca.push_back(pairs[k].first); cb.push_back(pairs[k].second);
			cs.push_back(PxU32(packed.size() / 8)); cc.push_back(cnt[k]);
			packed.insert(packed.end(), &cts[k * 64], &cts[k * 64] + 8 * cnt[k]);
			const float fa = friction[b0 + pairs[k].first];
			const float fb = pairs[k].second < n ? friction[b0 + pairs[k].second] : params[10];
			const float mu = (fa + fb) * 0.5f;
			mat.push_back(mu); mat.push_back(mu); mat.push_back(0.0f);
		}
		std::vector<float> vel(6 * size_t(n)), outPose(7 * size_t(n)), statics(7 * size_t(m) + 7);
		std::vector<PxU32> hs(2 * ca.size() + 2), hst(2 * ca.size() + 2), ord(ca.size() + 1);
		for(PxU32 k = 0; k < m; k++) memcpy(&statics[7 * k], staticPoses + 7 * size_t(s0 + k), 28);
		const float g[3] = {params[1], params[2], params[3]};
		if(ps)
		{
			tgsFrameRef(&rigid[b0], n, statics.data(), m, ca.data(), cb.data(), PxU32(ca.size()), cs.data(), cc.data(), packed.data(), mat.data(), g,
				dt, iterations[0], iterations[1], params[7], params[8], params[9], vel.data(), outPose.data(), hs.data(), hst.data(), ord.data(), NULL,
				NULL, ps->constraintAlloc, fptr.data(), fcount.data());
			for(size_t k = 0; k < cstate.size(); k++) { cstate[k]->frictions = fptr[k]; cstate[k]->nbFrictions = fcount[k]; }
		}
		else
			pxref_tgs_solve(&rigid[b0], n, statics.data(), m, ca.data(), cb.data(), PxU32(ca.size()), cs.data(), cc.data(), packed.data(), mat.data(), g,
				dt, iterations[0], iterations[1], params[7], params[8], params[9], vel.data(), outPose.data(), hs.data(), hst.data(), ord.data(), NULL, NULL);
		for(PxU32 i = 0; i < n; i++)
		{
			PxRigidBodyData& r = rigid[b0 + i];
			r.linearVelocity = PxVec3(vel[6 * i], vel[6 * i + 1], vel[6 * i + 2]);
			r.angularVelocity = PxVec3(vel[6 * i + 3], vel[6 * i + 4], vel[6 * i + 5]);
			r.body2World = PxTransform(PxVec3(outPose[7 * i + 4], outPose[7 * i + 5], outPose[7 * i + 6]),
				PxQuat(outPose[7 * i], outPose[7 * i + 1], outPose[7 * i + 2], outPose[7 * i + 3]));
		}
		b0 += n;
		s0 += m;
	}
	return 0;
}
} // namespace

// The reference's approximate reciprocal (aos::V3RecipFast, used by the box-box
// edge clipping in GuPCMContactBoxBox.cpp:140), four lanes at a time.
HX void pxref_recip_fast(const float* in, float* out, uint32_t n)
{
	using namespace physx::aos;
	for(uint32_t i = 0; i < n; i++)
	{
		const Vec3V v = V3Load(in[i]);
		const Vec3V r = V3RecipFast(v);
		FStore(V3GetX(r), &out[i]);
	}
}
