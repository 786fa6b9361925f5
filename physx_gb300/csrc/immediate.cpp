// libgbpx_immediate.so: the reference's immediate-mode entry points on the
// rigid-body path (physx/include/PxImmediateMode.h:267, 592-729) under their
// own C-linkage names, implemented on the GB300 through libgbpx's C ABI.  A
// program written against physx::immediate links these symbols from here.
//
// Each call moves the caller's arrays to the device and back (the reference's
// interface is host memory); many independent scenes should use gbpx_world_*
// instead.  What is not supported returns false / does nothing (see
// include/gbpx_immediate.h).
#include "gbpx.h"
#include "gbpx_immediate.h"

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

using namespace gbpx_px;

#define GX extern "C" __attribute__((visibility("default")))

namespace
{
const uint32_t NO_FACE_INDEX = 0xffffffffu;   // PXC_CONTACT_NO_FACE_INDEX

bool packShape(const PxGeometry& g, int& type, float* out)
{
	out[0] = out[1] = out[2] = out[3] = 0.0f;
	type = g.mType;
	switch(type)
	{
	case 0: out[0] = static_cast<const PxSphereGeometry&>(g).radius; return true;
	case 1: return true;
	case 2:
		out[0] = static_cast<const PxCapsuleGeometry&>(g).radius;
		out[1] = static_cast<const PxCapsuleGeometry&>(g).halfHeight;
		return true;
	case 3:
	{
		const PxVec3& h = static_cast<const PxBoxGeometry&>(g).halfExtents;
		out[0] = h.x; out[1] = h.y; out[2] = h.z;
		return true;
	}
	case 4:
	{
		// convex core: its type in bits 8..15, the first 3 core floats, the margin
		const PxConvexCoreGeometry& c = static_cast<const PxConvexCoreGeometry&>(g);
		if(c.mCoreType < 0 || c.mCoreType > 5) return false;
		type = 4 | (c.mCoreType << 8);
		memcpy(out, c.mCore, 3 * sizeof(float));
		out[3] = c.mMargin;
		return true;
	}
	default: return false;
	}
}

// PxConstraintBatchHeader::constraintType after constraint creation
// (lowleveldynamics/src/DySolverConstraintTypes.h:38, SolverConstraintType)
enum : uint16_t
{
	DY_SC_TYPE_RB_CONTACT = 1, DY_SC_TYPE_RB_1D = 2, DY_SC_TYPE_EXT_1D = 4, DY_SC_TYPE_STATIC_CONTACT = 5, DY_SC_TYPE_BLOCK_RB_CONTACT = 6,
	DY_SC_TYPE_BLOCK_STATIC_RB_CONTACT = 7, DY_SC_TYPE_BLOCK_1D = 8
};
bool isJointHeader(uint16_t type) { return type == DY_SC_TYPE_RB_1D || type == DY_SC_TYPE_EXT_1D || type == DY_SC_TYPE_BLOCK_1D; }

uint32_t stridesTotal(const PxConstraintBatchHeader* headers, uint32_t nbHeaders)
{
	uint32_t n = 0;
	for(uint32_t h = 0; h < nbHeaders; h++) n += headers[h].stride;
	return n;
}

// Contact manifold kept in a PxCache between calls: libgbpx's 288-byte record
// (opaque to the caller, who only hands the cache back), marked in its
// padding word so that a cache this library did not fill is taken as fresh.
constexpr uint32_t MANIFOLD_BYTES = 288;
constexpr uint32_t MANIFOLD_MAGIC_OFFSET = 76;
constexpr uint32_t MANIFOLD_USED_OFFSET = 68;
constexpr uint32_t MANIFOLD_MAGIC = 0x58504247u;
constexpr uint8_t CACHE_IS_MANIFOLD = 1;   // PxCache::mManifoldFlags of a single manifold

// does the pair kind keep a manifold (gEnablePCMCaching,
// physx/source/lowlevel/software/src/PxsContext.cpp:89): plane-capsule,
// plane-box, capsule-box, box-box
bool cachedKind(int t0, int t1)
{
	const int a = std::min(t0, t1), b = std::max(t0, t1);
	return (a == 1 && (b == 2 || b == 3)) || (a == 2 && b == 3) || (a == 3 && b == 3);
}

// Friction data a contact constraint leaves in the caller's friction memory
// (frictionPtr / frictionCount): libgbpx's 112-byte friction patches, whose
// first 16 bytes hold the body-0 normal and the broken flag (offset 12).
constexpr uint32_t PATCH_BYTES = 112;
constexpr uint32_t PATCH_BROKEN_OFFSET = 12;
constexpr uint32_t FRICTION_RECORD_BYTES = 16 + 4 * PATCH_BYTES;   // count, padding, 4 patches
constexpr uint32_t MAX_PATCHES = 4;

// Written after a constraint's rows in its constraint memory: where its
// friction patches are and which patch takes each row patch's broken flag.
struct RowTrailer
{
	uint8_t* friction;
	uint8_t slots[MAX_PATCHES];
	uint32_t count;
};
static_assert(sizeof(RowTrailer) == 16, "row trailer");

// PatchRows of libgbpx's constraint record (rows at +16, 48 bytes per patch,
// nbFriction at +44); record header: bodyA, bodyB, nbPatches, counts
uint32_t recordPatches(const uint8_t* rec) { uint32_t v; memcpy(&v, rec + 8, 4); return v; }
uint32_t recordPatchFriction(const uint8_t* rec, uint32_t p) { uint32_t v; memcpy(&v, rec + 16 + 48 * p + 44, 4); return v; }
} // namespace

// immediate::PxGenerateContacts.  The pair kinds whose contact manifold
// persists keep it in contactCache[i] (memory from the cache allocator, as the
// reference allocates it), the others leave the cache empty.
GX bool PxGenerateContacts(const PxGeometry* const* geom0, const PxGeometry* const* geom1, const PxTransform* pose0, const PxTransform* pose1,
                           PxCache* contactCache, uint32_t nbPairs, PxContactRecorder& contactRecorder, float contactDistance,
                           float meshContactMargin, float toleranceLength, PxCacheAllocator& allocator)
{
	if(!nbPairs) return true;
	if(!contactCache) return false;
	std::vector<int> t0(nbPairs), t1(nbPairs);
	std::vector<float> g0(4 * size_t(nbPairs)), g1(4 * size_t(nbPairs)), p0(7 * size_t(nbPairs)), p1(7 * size_t(nbPairs));
	for(uint32_t i = 0; i < nbPairs; i++)
	{
		if(!packShape(*geom0[i], t0[i], &g0[4 * size_t(i)]) || !packShape(*geom1[i], t1[i], &g1[4 * size_t(i)])) return false;
		memcpy(&p0[7 * size_t(i)], &pose0[i], 28);
		memcpy(&p1[7 * size_t(i)], &pose1[i], 28);
	}
	std::vector<float> out(size_t(nbPairs) * 4 * 8);
	std::vector<uint32_t> counts(nbPairs);
	std::vector<uint8_t> manifolds(size_t(nbPairs) * MANIFOLD_BYTES, 0);
	for(uint32_t i = 0; i < nbPairs; i++)
	{
		const PxCache& c = contactCache[i];
		if(c.mCachedData && c.mCachedSize == MANIFOLD_BYTES)
		{
			uint32_t magic;
			memcpy(&magic, c.mCachedData + MANIFOLD_MAGIC_OFFSET, 4);
			if(magic == MANIFOLD_MAGIC) memcpy(&manifolds[size_t(i) * MANIFOLD_BYTES], c.mCachedData, MANIFOLD_BYTES);
		}
	}
	if(gbpx_generate_contacts_cached(t0.data(), g0.data(), t1.data(), g1.data(), p0.data(), p1.data(), nbPairs, contactDistance,
	                                 meshContactMargin, toleranceLength, out.data(), 4, counts.data(), manifolds.data()) != GBPX_OK)
		return false;
	for(uint32_t i = 0; i < nbPairs; i++)
	{
		PxCache& c = contactCache[i];
		uint8_t* rec = &manifolds[size_t(i) * MANIFOLD_BYTES];
		uint32_t used;
		memcpy(&used, rec + MANIFOLD_USED_OFFSET, 4);
		uint8_t* mem = cachedKind(t0[i], t1[i]) && used ? allocator.allocateCacheData(MANIFOLD_BYTES) : nullptr;
		if(mem)
		{
			memcpy(rec + MANIFOLD_MAGIC_OFFSET, &MANIFOLD_MAGIC, 4);
			memcpy(mem, rec, MANIFOLD_BYTES);
			c.mCachedData = mem;
			c.mCachedSize = uint16_t(MANIFOLD_BYTES);
			c.mPairData = 0;
			c.mManifoldFlags = CACHE_IS_MANIFOLD;
		}
		else
		{
			c.mCachedData = nullptr;
			c.mCachedSize = 0;
			c.mPairData = 0;
			c.mManifoldFlags = 0;
		}
	}
	for(uint32_t i = 0; i < nbPairs; i++)
	{
		if(!counts[i]) continue;
		PxContactPoint cp[4];
		memset(cp, 0, sizeof(cp));
		for(uint32_t c = 0; c < counts[i]; c++)
		{
			const float* s = &out[(size_t(i) * 4 + c) * 8];
			cp[c].normal = PxVec3{s[0], s[1], s[2]};
			cp[c].separation = s[3];
			cp[c].point = PxVec3{s[4], s[5], s[6]};
			cp[c].internalFaceIndex1 = NO_FACE_INDEX;
		}
		contactRecorder.recordContacts(cp, counts[i], i);
	}
	return true;
}

GX void PxConstructSolverBodiesTGS(const PxRigidBodyData* inRigidData, PxTGSSolverBodyVel* outSolverBodyVel, PxTGSSolverBodyTxInertia* outSolverBodyTxInertia,
                                   PxTGSSolverBodyData* outSolverBodyData, uint32_t nbBodies, const PxVec3& gravity, float dt, bool gyroscopicForces)
{
	(void)gyroscopicForces;   // gyroscopic integration is not on this path
	gbpx_construct_solver_bodies_tgs(inRigidData, nbBodies, &gravity.x, dt, outSolverBodyVel, outSolverBodyTxInertia, outSolverBodyData);
}

GX void PxConstructStaticSolverBodyTGS(const PxTransform& globalPose, PxTGSSolverBodyVel& solverBodyVel, PxTGSSolverBodyTxInertia& solverBodyTxInertia,
                                       PxTGSSolverBodyData& solverBodyData)
{
	gbpx_construct_static_solver_bodies_tgs(&globalPose.q.x, 1, &solverBodyVel, &solverBodyTxInertia, &solverBodyData);
}

// PxBatchConstraintsTGS: bodies inside [solverBodies, solverBodies + nbBodies)
// are dynamic, every other body static or kinematic (as the reference).
GX uint32_t PxBatchConstraintsTGS(const PxSolverConstraintDesc* descs, uint32_t nbConstraints, PxTGSSolverBodyVel* solverBodies, uint32_t nbBodies,
                                  PxConstraintBatchHeader* outBatchHeaders, PxSolverConstraintDesc* outOrdered, void** articulations,
                                  uint32_t nbArticulations)
{
	(void)articulations;
	if(!nbConstraints || nbArticulations) return 0;
	std::vector<uint32_t> a(nbConstraints), b(nbConstraints), hs(nbConstraints), hst(nbConstraints), order(nbConstraints);
	auto index = [&](const PxTGSSolverBodyVel* p) {
		return (p >= solverBodies && p < solverBodies + nbBodies) ? uint32_t(p - solverBodies) : nbBodies;
	};
	for(uint32_t i = 0; i < nbConstraints; i++)
	{
		a[i] = index(descs[i].tgsBodyA);
		b[i] = index(descs[i].tgsBodyB);
	}
	// a header only joins constraints of one PxSolverConstraintDesc type (contact / joint)
	std::vector<uint8_t> kind(nbConstraints);
	for(uint32_t i = 0; i < nbConstraints; i++) kind[i] = uint8_t(descs[i].constraintLengthOver16);
	const uint32_t nbHeaders =
	    gbpx_batch_typed_constraints_tgs(a.data(), b.data(), kind.data(), nbConstraints, nbBodies, 1, hs.data(), hst.data(), order.data());
	for(uint32_t i = 0; i < nbConstraints; i++) outOrdered[i] = descs[order[i]];
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		outBatchHeaders[h].startIndex = hs[h];
		outBatchHeaders[h].stride = uint16_t(hst[h]);
		outBatchHeaders[h].constraintType = outOrdered[hs[h]].constraintLengthOver16;   // the descriptors' constraint type
	}
	return nbHeaders;
}

// PxCreateContactConstraintsTGS: rows per descriptor into the allocator's
// constraint memory (desc->constraint, desc->constraintLengthOver16).
GX bool PxCreateContactConstraintsTGS(PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, PxTGSSolverContactDesc* contactDescs,
                                      PxConstraintAllocator& allocator, float invDt, float invTotalDt, float bounceThreshold,
                                      float frictionOffsetThreshold, float correlationDistance)
{
	const uint32_t n = stridesTotal(batchHeaders, nbHeaders);
	if(!n) return true;
	static const PxTGSSolverBodyVel zeroVel = [] { PxTGSSolverBodyVel v; memset(&v, 0, sizeof(v)); v.isKinematic = true; return v; }();
	static const PxTGSSolverBodyTxInertia zeroTx = [] { PxTGSSolverBodyTxInertia t; memset(&t, 0, sizeof(t)); t.deltaBody2WorldQ.w = 1.0f; return t; }();
	static const PxTGSSolverBodyData zeroData = [] { PxTGSSolverBodyData d; memset(&d, 0, sizeof(d)); d.maxContactImpulse = 3.4e38f; return d; }();
	std::vector<PxTGSSolverBodyVel> v0(n), v1(n);
	std::vector<PxTGSSolverBodyTxInertia> x0(n), x1(n);
	std::vector<PxTGSSolverBodyData> d0(n), d1(n);
	std::vector<PxTransform> f0(n), f1(n);
	std::vector<uint32_t> cs(n), cc(n);
	std::vector<PxContactPoint> points;
	for(uint32_t k = 0; k < n; k++)
	{
		const PxTGSSolverContactDesc& d = contactDescs[k];
		if(!d.desc || d.numContacts > 4 || d.restDistance != 0.0f || d.hasMaxImpulse || d.invMassScales.linear0 != 1.0f || d.invMassScales.angular0 != 1.0f ||
		   d.invMassScales.linear1 != 1.0f || d.invMassScales.angular1 != 1.0f || (d.bodyState0 & eARTICULATION) || (d.bodyState1 & eARTICULATION))
			return false;
		v0[k] = d.body0 ? *d.body0 : zeroVel;
		v1[k] = d.body1 ? *d.body1 : zeroVel;
		if(d.bodyState0 != eDYNAMIC_BODY) v0[k].isKinematic = true;
		if(d.bodyState1 != eDYNAMIC_BODY) v1[k].isKinematic = true;
		x0[k] = d.body0TxI ? *d.body0TxI : zeroTx;
		x1[k] = d.body1TxI ? *d.body1TxI : zeroTx;
		d0[k] = d.bodyData0 ? *d.bodyData0 : zeroData;
		d1[k] = d.bodyData1 ? *d.bodyData1 : zeroData;
		f0[k] = d.bodyFrame0;
		f1[k] = d.bodyFrame1;
		cs[k] = uint32_t(points.size());
		cc[k] = d.numContacts;
		points.insert(points.end(), d.contacts, d.contacts + d.numContacts);
	}
	// a header of stride 4 with at most 64 contacts is built by the reference's
	// 4-wide block path (NpImmediateMode.cpp:1422-1444); isDynamic is per header
	std::vector<uint8_t> laneFlags(n, 0);
	for(uint32_t h = 0, k = 0; h < nbHeaders; k += batchHeaders[h].stride, h++)
	{
		if(batchHeaders[h].stride != 4) continue;
		uint32_t total = 0;
		bool dyn = false;
		for(uint32_t l = 0; l < 4; l++)
		{
			total += contactDescs[k + l].numContacts;
			dyn = dyn || contactDescs[k + l].bodyState1 == eDYNAMIC_BODY;
		}
		if(total > 64) continue;
		for(uint32_t l = 0; l < 4; l++)
			laneFlags[k + l] = uint8_t(1u | (dyn ? 2u : 0u) | (contactDescs[k + l].desc->bodyBDataIndex == 0 ? 4u : 0u));
	}
	// last frame's friction patches (frictionPtr / frictionCount)
	std::vector<uint8_t> frictionIn(size_t(n) * FRICTION_RECORD_BYTES, 0), frictionOut(size_t(n) * FRICTION_RECORD_BYTES, 0);
	for(uint32_t k = 0; k < n; k++)
	{
		const PxTGSSolverContactDesc& d = contactDescs[k];
		const uint32_t cnt = d.frictionPtr ? std::min<uint32_t>(d.frictionCount, MAX_PATCHES) : 0u;
		uint8_t* rec = &frictionIn[size_t(k) * FRICTION_RECORD_BYTES];
		memcpy(rec, &cnt, 4);
		if(cnt) memcpy(rec + 16, d.frictionPtr, size_t(cnt) * PATCH_BYTES);
	}
	const uint32_t stride = gbpx_constraint_row_stride();
	std::vector<uint8_t> rows(size_t(n) * stride);
	std::vector<uint32_t> bytes(n);
	if(gbpx_create_contact_constraints_tgs(n, v0.data(), v1.data(), x0.data(), x1.data(), d0.data(), d1.data(), &f0[0].q.x, &f1[0].q.x, cs.data(),
	                                       cc.data(), points.data(), uint32_t(points.size()), laneFlags.data(), frictionIn.data(),
	                                       frictionOut.data(), invDt, invTotalDt, bounceThreshold, frictionOffsetThreshold, correlationDistance,
	                                       rows.data(), bytes.data()) != GBPX_OK)
		return false;
	// header types as the reference leaves them (NpImmediateMode.cpp:1444-1472):
	// the 4-wide path's DY_SC_TYPE_BLOCK_RB_CONTACT / _BLOCK_STATIC_RB_CONTACT,
	// else the first constraint's DY_SC_TYPE_RB_CONTACT / _STATIC_CONTACT (a
	// static-typed header with a dynamic constraint becomes RB_CONTACT)
	for(uint32_t h = 0, k = 0; h < nbHeaders; k += batchHeaders[h].stride, h++)
	{
		PxConstraintBatchHeader& hd = batchHeaders[h];
		if(laneFlags[k] & 1u) { hd.constraintType = uint16_t((laneFlags[k] & 2u) ? DY_SC_TYPE_BLOCK_RB_CONTACT : DY_SC_TYPE_BLOCK_STATIC_RB_CONTACT); continue; }
		auto typeOf = [&](uint32_t j) {
			const int st = contactDescs[j].bodyState1;
			return uint16_t((st == eSTATIC_BODY || st == eKINEMATIC_BODY) ? DY_SC_TYPE_STATIC_CONTACT : DY_SC_TYPE_RB_CONTACT);
		};
		uint16_t type = typeOf(k);
		if(type == DY_SC_TYPE_STATIC_CONTACT)
			for(uint32_t l = 1; l < hd.stride; l++)
				if(typeOf(k + l) == DY_SC_TYPE_RB_CONTACT) { type = DY_SC_TYPE_RB_CONTACT; break; }
		hd.constraintType = type;
	}
	// header of every constraint (position of its header's first lane)
	std::vector<uint32_t> headerFirst(n, 0);
	for(uint32_t h = 0, k = 0; h < nbHeaders; k += batchHeaders[h].stride, h++)
		for(uint32_t l = 0; l < batchHeaders[h].stride; l++) headerFirst[k + l] = k;
	for(uint32_t k = 0; k < n; k++)
	{
		PxTGSSolverContactDesc& d = contactDescs[k];
		const uint32_t size = (bytes[k] + 15u) & ~15u;
		uint8_t* mem = allocator.reserveConstraintData(size + uint32_t(sizeof(RowTrailer)));
		if(!mem) return false;
		const uint8_t* rec = &rows[size_t(k) * stride];
		memcpy(mem, rec, size);
		d.desc->constraint = mem;
		d.desc->constraintLengthOver16 = uint16_t(size / 16);
		// the friction patches this constraint leaves, in the caller's friction memory
		const uint8_t* out = &frictionOut[size_t(k) * FRICTION_RECORD_BYTES];
		uint32_t cnt;
		memcpy(&cnt, out, 4);
		cnt = std::min<uint32_t>(cnt, MAX_PATCHES);
		uint8_t* fmem = cnt ? allocator.reserveFrictionData(cnt * PATCH_BYTES) : nullptr;
		if(cnt && !fmem) return false;
		if(fmem) memcpy(fmem, out + 16, size_t(cnt) * PATCH_BYTES);
		d.frictionPtr = fmem;
		d.frictionCount = uint8_t(cnt);
		d.numFrictionPatches = cnt;
		// broken-flag slot of each row patch: the patch itself, or for a block
		// lane the header's earlier patch rows that had friction in any lane
		// (DyTGSContactPrepBlock.cpp:1218-1222)
		RowTrailer tr;
		memset(&tr, 0, sizeof(tr));
		tr.friction = fmem;
		tr.count = cnt;
		const uint32_t np = std::min<uint32_t>(recordPatches(rec), MAX_PATCHES);
		const bool block = laneFlags[k] & 1u;
		for(uint32_t p = 0; p < np; p++)
		{
			uint32_t slot = p;
			if(block)
			{
				slot = 0;
				for(uint32_t j = 0; j < p; j++)
				{
					bool any = false;
					for(uint32_t l = 0; l < 4; l++)
					{
						const uint8_t* r2 = &rows[size_t(headerFirst[k] + l) * stride];
						if(j < recordPatches(r2) && recordPatchFriction(r2, j) > 0) any = true;
					}
					if(any) slot++;
				}
			}
			tr.slots[p] = uint8_t(slot);
		}
		memcpy(mem + size, &tr, sizeof(tr));
	}
	return true;
}

// Joint records in constraint memory: the record header (up to its rows) and
// the rows in use, this library's format (gbpx_joint_record_bytes() at most).
constexpr uint32_t JOINT_HEADER_BYTES = 192, JOINT_ROW_BYTES = 96, JOINT_COUNT_OFFSET = 8;
uint32_t jointRecordUsedBytes(const uint8_t* rec)
{
	uint32_t count;
	memcpy(&count, rec + JOINT_COUNT_OFFSET, 4);
	return JOINT_HEADER_BYTES + std::min<uint32_t>(count, 12) * JOINT_ROW_BYTES;
}

// Dy::ConstraintWriteback (lowleveldynamics/include/DyConstraintWriteBack.h:42)
struct JointWriteback
{
	PxVec3 linearImpulse;
	uint32_t brokenAndResidual;   // broken in bit 31 (setCombined), position residual (0) below
	PxVec3 angularImpulse;
	float residual;
};

// PxCreateJointConstraintsTGS: one record per joint into the allocator's
// constraint memory; a header of stride 4 whose joints all have rows takes the
// reference's 4-wide path (NpImmediateMode.cpp:1495-1517) and is typed
// DY_SC_TYPE_BLOCK_1D, every other DY_SC_TYPE_RB_1D.  A joint without rows gets
// no constraint (desc->constraint = null).  The caller's rows are read, not
// rewritten.  Joints between articulation links and eIMPROVED_SLERP drives are
// not supported (false).
GX bool PxCreateJointConstraintsTGS(PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, PxTGSSolverConstraintPrepDesc* jointDescs,
                                    PxConstraintAllocator& allocator, float dt, float totalDt, float invDt, float invTotalDt, float lengthScale)
{
	const uint32_t n = stridesTotal(batchHeaders, nbHeaders);
	if(!n) return true;
	if(!(dt > 0.0f) || !(totalDt > 0.0f)) return false;
	static const PxTGSSolverBodyVel zeroVel = [] { PxTGSSolverBodyVel v; memset(&v, 0, sizeof(v)); v.isKinematic = true; return v; }();
	static const PxTGSSolverBodyTxInertia zeroTx = [] { PxTGSSolverBodyTxInertia t; memset(&t, 0, sizeof(t)); t.deltaBody2WorldQ.w = 1.0f; return t; }();
	static const PxTGSSolverBodyData zeroData = [] { PxTGSSolverBodyData d; memset(&d, 0, sizeof(d)); d.maxContactImpulse = 3.4e38f; return d; }();
	std::vector<PxTGSSolverBodyVel> v0(n), v1(n);
	std::vector<PxTGSSolverBodyTxInertia> x0(n), x1(n);
	std::vector<PxTGSSolverBodyData> d0(n), d1(n);
	std::vector<PxTransform> f0(n), f1(n);
	std::vector<uint32_t> rs(n), rc(n);
	std::vector<Px1DConstraint> rows;
	std::vector<float> params(size_t(n) * 20, 0.0f);
	std::vector<uint8_t> block(n, 0);
	for(uint32_t k = 0; k < n; k++)
	{
		const PxTGSSolverConstraintPrepDesc& d = jointDescs[k];
		if(!d.desc || d.numRows > 12 || (d.numRows && !d.rows) || d.improvedSlerp || (d.bodyState0 & eARTICULATION) || (d.bodyState1 & eARTICULATION))
			return false;
		v0[k] = d.body0 ? *d.body0 : zeroVel;
		v1[k] = d.body1 ? *d.body1 : zeroVel;
		x0[k] = d.body0TxI ? *d.body0TxI : zeroTx;
		x1[k] = d.body1TxI ? *d.body1TxI : zeroTx;
		d0[k] = d.bodyData0 ? *d.bodyData0 : zeroData;
		d1[k] = d.bodyData1 ? *d.bodyData1 : zeroData;
		f0[k] = d.bodyFrame0;
		f1[k] = d.bodyFrame1;
		rs[k] = uint32_t(rows.size());
		rc[k] = d.numRows;
		rows.insert(rows.end(), d.rows, d.rows + d.numRows);
		float* p = &params[size_t(k) * 20];
		p[0] = d.invMassScales.linear0; p[1] = d.invMassScales.angular0; p[2] = d.invMassScales.linear1; p[3] = d.invMassScales.angular1;
		p[4] = d.cA2w.v.x; p[5] = d.cA2w.v.y; p[6] = d.cA2w.v.z;
		p[7] = d.cB2w.v.x; p[8] = d.cB2w.v.y; p[9] = d.cB2w.v.z;
		p[10] = d.body0WorldOffset.v.x; p[11] = d.body0WorldOffset.v.y; p[12] = d.body0WorldOffset.v.z;
		p[13] = d.linBreakForce; p[14] = d.angBreakForce; p[15] = d.minResponseThreshold;
		p[16] = float((d.disablePreprocessing ? 1u : 0u) | (d.driveLimitsAreForces ? 4u : 0u));
	}
	for(uint32_t h = 0, k = 0; h < nbHeaders; k += batchHeaders[h].stride, h++)
	{
		PxConstraintBatchHeader& hd = batchHeaders[h];
		bool b = hd.stride == 4;
		for(uint32_t l = 0; l < hd.stride && b; l++) b = jointDescs[k + l].numRows > 0;
		hd.constraintType = b ? DY_SC_TYPE_BLOCK_1D : DY_SC_TYPE_RB_1D;
		for(uint32_t l = 0; l < hd.stride; l++) block[k + l] = b ? 1 : 0;
	}
	const uint32_t recBytes = gbpx_joint_record_bytes();
	std::vector<uint8_t> recs(size_t(n) * recBytes);
	if(gbpx_create_joint_constraints_tgs(n, v0.data(), v1.data(), x0.data(), x1.data(), d0.data(), d1.data(), &f0[0].q.x, &f1[0].q.x, rs.data(),
	                                     rc.data(), rows.data(), uint32_t(rows.size()), params.data(), block.data(), dt, totalDt, invDt, invTotalDt,
	                                     lengthScale, recs.data()) != GBPX_OK)
		return false;
	for(uint32_t k = 0; k < n; k++)
	{
		PxSolverConstraintDesc& sd = *jointDescs[k].desc;
		if(jointDescs[k].numRows == 0)
		{
			sd.constraint = nullptr;
			sd.writeBack = nullptr;
			sd.constraintLengthOver16 = 0;
			continue;
		}
		const uint8_t* rec = &recs[size_t(k) * recBytes];
		const uint32_t size = jointRecordUsedBytes(rec);
		uint8_t* mem = allocator.reserveConstraintData(size);
		if(!mem) return false;
		memcpy(mem, rec, size);
		sd.constraint = mem;
		sd.constraintLengthOver16 = uint16_t(size / 16);
		sd.writeBack = jointDescs[k].writeback;
	}
	return true;
}

// PxSolveConstraintsTGS: headers are solved in order; consecutive headers whose
// constraints touch distinct dynamic bodies run as one parallel wave.  Joint
// headers (DY_SC_TYPE_RB_1D / _BLOCK_1D) hold joint records, every other
// header contact rows.
GX void PxSolveConstraintsTGS(const PxConstraintBatchHeader* batchHeaders, uint32_t nbBatchHeaders, const PxSolverConstraintDesc* descs,
                              PxTGSSolverBodyVel* solverBodies, PxTGSSolverBodyTxInertia* txInertias, uint32_t nbSolverBodies, uint32_t nbPositionIterations,
                              uint32_t nbVelocityIterations, float dt, float invDt, uint32_t nbSolverArticulations, void** solverArticulations, void* Z,
                              void* deltaV)
{
	(void)invDt;
	(void)solverArticulations;
	(void)Z;
	(void)deltaV;
	if(nbSolverArticulations || !nbSolverBodies) return;
	// bodies: the caller's solver bodies, then every other (static / kinematic) body the constraints reference
	std::vector<PxTGSSolverBodyVel> vel(solverBodies, solverBodies + nbSolverBodies);
	std::vector<PxTGSSolverBodyTxInertia> tx(txInertias, txInertias + nbSolverBodies);
	std::unordered_map<const PxTGSSolverBodyVel*, uint32_t> extra;
	PxTGSSolverBodyTxInertia zeroTx;
	memset(&zeroTx, 0, sizeof(zeroTx));
	zeroTx.deltaBody2WorldQ.w = 1.0f;
	auto index = [&](const PxTGSSolverBodyVel* p) -> uint32_t {
		if(p >= solverBodies && p < solverBodies + nbSolverBodies) return uint32_t(p - solverBodies);
		auto it = extra.find(p);
		if(it != extra.end()) return it->second;
		const uint32_t id = uint32_t(vel.size());
		extra[p] = id;
		vel.push_back(*p);
		tx.push_back(zeroTx);
		return id;
	};
	const uint32_t stride = gbpx_constraint_row_stride();
	const uint32_t jointBytes = gbpx_joint_record_bytes();
	std::vector<uint8_t> rows, joints;
	std::vector<uint32_t> a, b, ja, jb, waveEnds, jointWaveEnds;
	std::vector<const PxSolverConstraintDesc*> contactDesc, jointDesc;
	std::vector<uint32_t> lastWave(nbSolverBodies, 0);   // per dynamic body: wave that last used it (+1)
	uint32_t wave = 1;
	bool waveOpen = false;
	for(uint32_t h = 0; h < nbBatchHeaders; h++)
	{
		const PxConstraintBatchHeader& hd = batchHeaders[h];
		const bool isJoint = isJointHeader(hd.constraintType);
		bool clash = false;
		for(uint32_t j = 0; j < hd.stride; j++)
		{
			const PxSolverConstraintDesc& d = descs[hd.startIndex + j];
			const uint32_t ia = index(d.tgsBodyA), ib = index(d.tgsBodyB);
			clash = clash || (ia < nbSolverBodies && lastWave[ia] == wave) || (ib < nbSolverBodies && lastWave[ib] == wave);
		}
		if(clash && waveOpen)
		{
			waveEnds.push_back(uint32_t(a.size()));
			jointWaveEnds.push_back(uint32_t(ja.size()));
			wave++;
		}
		for(uint32_t j = 0; j < hd.stride; j++)
		{
			const PxSolverConstraintDesc& d = descs[hd.startIndex + j];
			const uint32_t ia = index(d.tgsBodyA), ib = index(d.tgsBodyB);
			if(ia < nbSolverBodies) lastWave[ia] = wave;
			if(ib < nbSolverBodies) lastWave[ib] = wave;
			if(isJoint)
			{
				if(!d.constraint) continue;   // a joint without rows
				ja.push_back(ia);
				jb.push_back(ib);
				jointDesc.push_back(&d);
				joints.resize(joints.size() + jointBytes, 0);
				memcpy(&joints[joints.size() - jointBytes], d.constraint, std::min<size_t>(size_t(d.constraintLengthOver16) * 16, jointBytes));
			}
			else
			{
				a.push_back(ia);
				b.push_back(ib);
				contactDesc.push_back(&d);
				rows.resize(rows.size() + stride, 0);
				if(d.constraint) memcpy(&rows[rows.size() - stride], d.constraint, std::min<size_t>(size_t(d.constraintLengthOver16) * 16, stride));
			}
		}
		waveOpen = true;
	}
	const uint32_t n = uint32_t(a.size()), nj = uint32_t(ja.size());
	if(waveOpen)
	{
		waveEnds.push_back(n);
		jointWaveEnds.push_back(nj);
	}
	std::vector<uint32_t> broken(n ? n : 1, 0), jointBroken(nj ? nj : 1, 0);
	std::vector<float> jointForce(size_t(nj ? nj : 1) * 6, 0.0f);
	if(gbpx_solve_constraints_joints_tgs(n ? rows.data() : nullptr, a.data(), b.data(), n, waveEnds.data(), nj ? joints.data() : nullptr, ja.data(),
	                                     jb.data(), nj, jointWaveEnds.data(), uint32_t(waveEnds.size()), vel.data(), tx.data(), uint32_t(vel.size()),
	                                     nbSolverBodies, nbPositionIterations, nbVelocityIterations, dt, broken.data(), jointForce.data(),
	                                     jointBroken.data()) != GBPX_OK)
		return;
	memcpy(solverBodies, vel.data(), size_t(nbSolverBodies) * sizeof(PxTGSSolverBodyVel));
	memcpy(txInertias, tx.data(), size_t(nbSolverBodies) * sizeof(PxTGSSolverBodyTxInertia));
	for(uint32_t k = 0; k < n; k++)
	{
		const PxSolverConstraintDesc& d = *contactDesc[k];
		if(!d.constraint) continue;
		const size_t size = size_t(d.constraintLengthOver16) * 16;
		memcpy(d.constraint, &rows[size_t(k) * stride], std::min<size_t>(size, stride));
		// write-back of the last iteration: clamped friction marks its patch broken
		if(broken[k])
		{
			RowTrailer tr;
			memcpy(&tr, d.constraint + size, sizeof(tr));
			for(uint32_t p = 0; p < MAX_PATCHES; p++)
				if((broken[k] & (1u << p)) && tr.friction && tr.slots[p] < tr.count)
				{
					const uint32_t one = 1;
					memcpy(tr.friction + size_t(tr.slots[p]) * PATCH_BYTES + PATCH_BROKEN_OFFSET, &one, 4);
				}
		}
	}
	// joints: records back into constraint memory, impulses and broken flags to the write-back
	for(uint32_t k = 0; k < nj; k++)
	{
		const PxSolverConstraintDesc& d = *jointDesc[k];
		memcpy(d.constraint, &joints[size_t(k) * jointBytes], std::min<size_t>(size_t(d.constraintLengthOver16) * 16, jointBytes));
		if(d.writeBack)
		{
			JointWriteback w;
			const float* f = &jointForce[size_t(k) * 6];
			w.linearImpulse = PxVec3{f[0], f[1], f[2]};
			w.angularImpulse = PxVec3{f[3], f[4], f[5]};
			w.brokenAndResidual = jointBroken[k] ? 0x80000000u : 0u;
			w.residual = 0.0f;
			memcpy(d.writeBack, &w, sizeof(w));
		}
	}
}

GX void PxIntegrateSolverBodiesTGS(PxTGSSolverBodyVel* solverBody, const PxTGSSolverBodyTxInertia* txInertia, PxTransform* poses, uint32_t nbBodiesToIntegrate,
                                   float dt)
{
	(void)dt;
	gbpx_integrate_solver_bodies_tgs(solverBody, txInertia, &poses[0].q.x, nbBodiesToIntegrate);
}

// ------------------------------------------------------------------ PGS
// PxConstructSolverBodies / PxConstructStaticSolverBody / PxBatchConstraints /
// PxCreateContactConstraints / PxSolveConstraints / PxIntegrateSolverBodies
// (physx/include/PxImmediateMode.h:111-245) over libgbpx's PGS stages.  The
// constraint memory of a contact descriptor holds libgbpx's PGS record; body
// indices are resolved at the solve from the descriptors' PxSolverBody pointers.
GX void PxConstructSolverBodies(const PxRigidBodyData* inRigidData, PxSolverBodyData* outSolverBodyData, uint32_t nbBodies, const PxVec3& gravity,
                                float dt, bool gyroscopicForces)
{
	(void)gyroscopicForces;   // gyroscopic integration is not on this path
	gbpx_construct_solver_bodies_pgs(inRigidData, nullptr, nbBodies, &gravity.x, dt, outSolverBodyData);
}

GX void PxConstructStaticSolverBody(const PxTransform& globalPose, PxSolverBodyData& solverBodyData)
{
	gbpx_construct_solver_bodies_pgs(nullptr, &globalPose.q.x, 1, nullptr, 0.0f, &solverBodyData);
}

// PxBatchConstraints: bodies inside [solverBodies, solverBodies + nbBodies)
// are dynamic, every other body static or kinematic (as the reference).
GX uint32_t PxBatchConstraints(const PxSolverConstraintDesc* descs, uint32_t nbConstraints, PxSolverBody* solverBodies, uint32_t nbBodies,
                               PxConstraintBatchHeader* outBatchHeaders, PxSolverConstraintDesc* outOrdered, void** articulations,
                               uint32_t nbArticulations)
{
	(void)articulations;
	if(!nbConstraints || nbArticulations) return 0;
	std::vector<uint32_t> a(nbConstraints), b(nbConstraints), hs(nbConstraints), hst(nbConstraints), order(nbConstraints);
	auto index = [&](const PxSolverBody* p) { return (p >= solverBodies && p < solverBodies + nbBodies) ? uint32_t(p - solverBodies) : nbBodies; };
	for(uint32_t i = 0; i < nbConstraints; i++)
	{
		a[i] = index(descs[i].bodyA);
		b[i] = index(descs[i].bodyB);
	}
	std::vector<uint8_t> kind(nbConstraints);
	for(uint32_t i = 0; i < nbConstraints; i++) kind[i] = uint8_t(descs[i].constraintLengthOver16);
	const uint32_t nbHeaders =
	    gbpx_batch_typed_constraints_tgs(a.data(), b.data(), kind.data(), nbConstraints, nbBodies, 1, hs.data(), hst.data(), order.data());
	for(uint32_t i = 0; i < nbConstraints; i++) outOrdered[i] = descs[order[i]];
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		outBatchHeaders[h].startIndex = hs[h];
		outBatchHeaders[h].stride = uint16_t(hst[h]);
		outBatchHeaders[h].constraintType = outOrdered[hs[h]].constraintLengthOver16;
	}
	return nbHeaders;
}

// PxCreateJointConstraintsWithImmediateShadersTGS (NpImmediateMode.cpp:1543-1628):
// each descriptor's shader fills its rows on the host (unit mass scales and a
// zero body-0 offset first, up to 20 rows set to zero with unbounded impulse
// limits, as setupConstraintRows, DyConstraintPrep.h:115), then the rows of
// every header are prepared on the device in one PxCreateJointConstraintsTGS
// call.  The reference prepares header by header into one reused row buffer;
// each shader sees the same fresh rows here.
GX bool PxCreateJointConstraintsWithImmediateShadersTGS(PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, PxImmediateConstraint* constraints,
                                                        PxTGSSolverConstraintPrepDesc* jointDescs, PxConstraintAllocator& allocator, float dt,
                                                        float totalDt, float invDt, float invTotalDt, float lengthScale)
{
	constexpr uint32_t MAX_ROWS = 20;   // Dy::MAX_CONSTRAINT_ROWS
	const uint32_t n = stridesTotal(batchHeaders, nbHeaders);
	if(!n) return true;
	if(!constraints || !jointDescs) return false;
	std::vector<Px1DConstraint> rows(size_t(n) * MAX_ROWS);
	uint32_t d = 0;
	for(uint32_t h = 0; h < nbHeaders; h++)
		for(uint32_t a = 0; a < batchHeaders[h].stride; a++, d++)
		{
			PxTGSSolverConstraintPrepDesc& desc = jointDescs[d];
			const PxImmediateConstraint& ic = constraints[d];
			if(!ic.prep) return false;
			Px1DConstraint* r = rows.data() + size_t(d) * MAX_ROWS;
			memset(r, 0, sizeof(Px1DConstraint) * MAX_ROWS);
			for(uint32_t i = 0; i < MAX_ROWS; i++)
			{
				r[i].minImpulse = -3.402823466e+38f;
				r[i].maxImpulse = 3.402823466e+38f;
			}
			desc.invMassScales = PxConstraintInvMassScale{1.0f, 1.0f, 1.0f, 1.0f};
			desc.body0WorldOffset.v = PxVec3{0.0f, 0.0f, 0.0f};
			const uint32_t count = ic.prep(r, desc.body0WorldOffset, MAX_ROWS, desc.invMassScales, ic.constantBlock, desc.bodyFrame0, desc.bodyFrame1,
			                               false, desc.cA2w, desc.cB2w);
			if(count > MAX_ROWS) return false;
			desc.rows = r;
			desc.numRows = count;
		}
	return PxCreateJointConstraintsTGS(batchHeaders, nbHeaders, jointDescs, allocator, dt, totalDt, invDt, invTotalDt, lengthScale);
}

// PxCreateContactConstraints: a record per descriptor into the allocator's
// constraint memory; the header types as the reference leaves them
// (NpImmediateMode.cpp:292-367).  Friction data is not kept between frames.
GX bool PxCreateContactConstraints(PxConstraintBatchHeader* batchHeaders, uint32_t nbHeaders, PxSolverContactDesc* contactDescs,
                                   PxConstraintAllocator& allocator, float invDt, float bounceThreshold, float frictionOffsetThreshold,
                                   float correlationDistance, void* ZV)
{
	(void)correlationDistance;
	(void)ZV;
	const uint32_t n = stridesTotal(batchHeaders, nbHeaders);
	if(!n) return true;
	static const PxSolverBodyData zeroData = [] {
		PxSolverBodyData d;
		memset(&d, 0, sizeof(d));
		d.maxContactImpulse = 3.4e38f;
		d.penBiasClamp = -3.4e38f;
		d.body2World.q.w = 1.0f;
		return d;
	}();
	std::vector<PxSolverBodyData> d0(n), d1(n);
	std::vector<PxTransform> f0(n), f1(n);
	std::vector<uint32_t> cs(n), cc(n);
	std::vector<PxContactPoint> points;
	for(uint32_t k = 0; k < n; k++)
	{
		const PxSolverContactDesc& d = contactDescs[k];
		if(!d.desc || !d.numContacts || d.numContacts > 4 || d.restDistance != 0.0f || d.hasMaxImpulse || d.invMassScales.linear0 != 1.0f ||
		   d.invMassScales.angular0 != 1.0f || d.invMassScales.linear1 != 1.0f || d.invMassScales.angular1 != 1.0f || d.bodyState0 != eDYNAMIC_BODY ||
		   (d.bodyState1 & eARTICULATION))
			return false;
		d0[k] = d.data0 ? *d.data0 : zeroData;
		d1[k] = d.data1 ? *d.data1 : zeroData;
		f0[k] = d.bodyFrame0;
		f1[k] = d.bodyFrame1;
		cs[k] = uint32_t(points.size());
		cc[k] = d.numContacts;
		points.insert(points.end(), d.contacts, d.contacts + d.numContacts);
	}
	// a header of stride 4 with at most 64 contacts takes the reference's 4-wide
	// block path (NpImmediateMode.cpp:312-330); otherwise the first constraint's
	// type, a static one turning dynamic when another constraint of the header is
	std::vector<uint8_t> laneFlags(n, 0);
	for(uint32_t h = 0, k = 0; h < nbHeaders; k += batchHeaders[h].stride, h++)
	{
		PxConstraintBatchHeader& hd = batchHeaders[h];
		uint32_t total = 0;
		bool dyn = false;
		for(uint32_t l = 0; l < hd.stride; l++)
		{
			total += contactDescs[k + l].numContacts;
			dyn = dyn || contactDescs[k + l].bodyState1 == eDYNAMIC_BODY;
		}
		if(hd.stride == 4 && total <= 64)
		{
			hd.constraintType = uint16_t(dyn ? DY_SC_TYPE_BLOCK_RB_CONTACT : DY_SC_TYPE_BLOCK_STATIC_RB_CONTACT);
			for(uint32_t l = 0; l < 4; l++)
				laneFlags[k + l] = uint8_t(1u | (dyn ? 2u : 0u) | (contactDescs[k + l].desc->bodyBDataIndex != 0 ? 4u : 0u));
			continue;
		}
		auto typeOf = [&](uint32_t j) {
			const int st = contactDescs[j].bodyState1;
			return uint16_t((st == eSTATIC_BODY || st == eKINEMATIC_BODY) ? DY_SC_TYPE_STATIC_CONTACT : DY_SC_TYPE_RB_CONTACT);
		};
		uint16_t type = typeOf(k);
		if(type == DY_SC_TYPE_STATIC_CONTACT)
			for(uint32_t l = 1; l < hd.stride; l++)
				if(typeOf(k + l) == DY_SC_TYPE_RB_CONTACT) { type = DY_SC_TYPE_RB_CONTACT; break; }
		hd.constraintType = type;
		for(uint32_t l = 0; l < hd.stride; l++) laneFlags[k + l] = type == DY_SC_TYPE_RB_CONTACT ? 8u : 0u;
	}
	const uint32_t recBytes = gbpx_pgs_record_bytes();
	std::vector<uint8_t> recs(size_t(n) * recBytes);
	if(gbpx_create_contact_constraints_pgs(n, d0.data(), d1.data(), &f0[0].q.x, &f1[0].q.x, cs.data(), cc.data(), points.data(),
	                                       uint32_t(points.size()), laneFlags.data(), invDt, bounceThreshold, frictionOffsetThreshold,
	                                       recs.data()) != GBPX_OK)
		return false;
	for(uint32_t k = 0; k < n; k++)
	{
		PxSolverContactDesc& d = contactDescs[k];
		uint8_t* mem = allocator.reserveConstraintData(recBytes);
		if(!mem) return false;
		memcpy(mem, &recs[size_t(k) * recBytes], recBytes);
		d.desc->constraint = mem;
		d.desc->constraintLengthOver16 = uint16_t(recBytes / 16);
		d.desc->writeBack = d.contactForces;
		d.frictionPtr = nullptr;
		d.frictionCount = 0;
	}
	return true;
}

// PxSolveConstraints: headers are solved in order; consecutive headers whose
// constraints touch distinct dynamic bodies run as one parallel wave.  The
// normal impulses of the last velocity iteration go to each descriptor's
// write-back (its PxSolverContactDesc::contactForces), in row order.
GX void PxSolveConstraints(const PxConstraintBatchHeader* batchHeaders, uint32_t nbBatchHeaders, const PxSolverConstraintDesc* descs,
                           const PxSolverBody* solverBodies, PxVec3* linearMotionVelocity, PxVec3* angularMotionVelocity, uint32_t nbSolverBodies,
                           uint32_t nbPositionIterations, uint32_t nbVelocityIterations, float dt, float invDt, uint32_t nbSolverArticulations,
                           void** solverArticulations, void* Z, void* deltaV)
{
	(void)dt;
	(void)invDt;
	(void)solverArticulations;
	(void)Z;
	(void)deltaV;
	if(nbSolverArticulations || !nbSolverBodies || !nbPositionIterations || !nbVelocityIterations) return;
	auto index = [&](const PxSolverBody* p) {
		return (p >= solverBodies && p < solverBodies + nbSolverBodies) ? uint32_t(p - solverBodies) : nbSolverBodies;
	};
	const uint32_t recBytes = gbpx_pgs_record_bytes();
	std::vector<uint8_t> recs;
	std::vector<uint32_t> a, b, waveEnds;
	std::vector<const PxSolverConstraintDesc*> used;
	std::vector<uint32_t> lastWave(nbSolverBodies, 0);
	uint32_t wave = 1;
	bool waveOpen = false;
	for(uint32_t h = 0; h < nbBatchHeaders; h++)
	{
		const PxConstraintBatchHeader& hd = batchHeaders[h];
		if(isJointHeader(hd.constraintType)) return;   // PGS joints are not on this path
		bool clash = false;
		for(uint32_t j = 0; j < hd.stride; j++)
		{
			const PxSolverConstraintDesc& d = descs[hd.startIndex + j];
			const uint32_t ia = index(d.bodyA), ib = index(d.bodyB);
			clash = clash || (ia < nbSolverBodies && lastWave[ia] == wave) || (ib < nbSolverBodies && lastWave[ib] == wave);
		}
		if(clash && waveOpen)
		{
			waveEnds.push_back(uint32_t(a.size()));
			wave++;
		}
		for(uint32_t j = 0; j < hd.stride; j++)
		{
			const PxSolverConstraintDesc& d = descs[hd.startIndex + j];
			const uint32_t ia = index(d.bodyA), ib = index(d.bodyB);
			if(ia < nbSolverBodies) lastWave[ia] = wave;
			if(ib < nbSolverBodies) lastWave[ib] = wave;
			if(!d.constraint) continue;
			a.push_back(ia);
			b.push_back(ib);
			used.push_back(&d);
			recs.resize(recs.size() + recBytes);
			memcpy(&recs[recs.size() - recBytes], d.constraint, recBytes);
		}
		waveOpen = true;
	}
	const uint32_t n = uint32_t(a.size());
	if(waveOpen) waveEnds.push_back(n);
	std::vector<PxSolverBody> bodies(solverBodies, solverBodies + nbSolverBodies);
	if(gbpx_solve_constraints_pgs(n ? recs.data() : nullptr, a.data(), b.data(), n, waveEnds.data(), uint32_t(waveEnds.size()), bodies.data(),
	                              nbSolverBodies, nbPositionIterations, nbVelocityIterations, &linearMotionVelocity[0].x,
	                              &angularMotionVelocity[0].x) != GBPX_OK)
		return;
	// PxSolveConstraints leaves the velocities in the caller's solver bodies
	memcpy(const_cast<PxSolverBody*>(solverBodies), bodies.data(), size_t(nbSolverBodies) * sizeof(PxSolverBody));
	for(uint32_t k = 0; k < n; k++)
	{
		const PxSolverConstraintDesc& d = *used[k];
		const uint8_t* rec = &recs[size_t(k) * recBytes];
		memcpy(d.constraint, rec, recBytes);
		if(!d.writeBack) continue;
		// record: bodyA, bodyB, nbPatches, flags, 4 patches of 48 bytes (nbPoints at +36),
		// then the point rows (48 bytes, the impulse at +40)
		uint32_t nbPatches;
		memcpy(&nbPatches, rec + 8, 4);
		uint32_t points = 0;
		for(uint32_t p = 0; p < std::min<uint32_t>(nbPatches, 4); p++)
		{
			uint32_t np;
			memcpy(&np, rec + 16 + 48 * p + 36, 4);
			points += np;
		}
		float* out = static_cast<float*>(d.writeBack);
		for(uint32_t i = 0; i < std::min<uint32_t>(points, 4); i++) memcpy(&out[i], rec + 16 + 4 * 48 + 48 * i + 40, 4);
	}
}

GX void PxIntegrateSolverBodies(PxSolverBodyData* solverBodyData, PxSolverBody* solverBody, PxVec3* linearMotionVelocity, PxVec3* angularMotionState,
                                uint32_t nbBodiesToIntegrate, float dt)
{
	gbpx_integrate_solver_bodies_pgs(solverBodyData, solverBody, &linearMotionVelocity[0].x, &angularMotionState[0].x, nbBodiesToIntegrate, dt);
}

// ------------------------------------------------------------------ broadphase
// PxCreateBroadPhase / PxBroadPhase (physx/include/PxBroadPhase.h:492-629) and
// PxCreateAABBManager / PxAABBManager (:642-796) over libgbpx's ABP-compatible
// broadphase (gbpx_bp_*).
namespace
{
// Page-locked host memory: user bounds, groups and distances allocated here
// reach the device without a staging copy.
struct PinnedAllocator : PxAllocatorCallback
{
	void* allocate(size_t size, const char*, const char*, int) override
	{
		void* p = nullptr;
		return gbpx_host_alloc(size ? size : 1, &p) == GBPX_OK ? p : nullptr;
	}
	void deallocate(void* ptr) override { if(ptr) gbpx_host_free(ptr); }
};
PinnedAllocator gPinned;

class GbpxBroadPhase : public PxBroadPhase
{
public:
	GbpxBroadPhase(const PxBroadPhaseDesc& d, void* h) : desc(d), handle(h) {}
	void release() override
	{
		if(manager) return;   // the reference refuses while an AABB manager is attached
		gbpx_bp_release(handle);
		delete this;
	}
	PxBroadPhaseType::Enum getType() const override { return desc.mType; }
	void getCaps(PxBroadPhaseCaps& caps) const override { caps.mMaxNbRegions = 0; }
	PxBroadPhaseRegions* getRegions() override { return nullptr; }
	PxAllocatorCallback* getAllocator() override { return &gPinned; }
	uint64_t getContextID() const override { return desc.mContextID; }
	void setScratchBlock(void*, uint32_t) override {}
	void update(const PxBroadPhaseUpdateData& u, PxBaseTask*) override
	{
		status = gbpx_bp_update(handle, u.mCreated, u.mNbCreated, u.mUpdated, u.mNbUpdated, u.mRemoved, u.mNbRemoved,
		                        reinterpret_cast<const float*>(u.mBounds), u.mGroups, u.mDistances, u.mCapacity);
	}
	void fetchResults(PxBroadPhaseResults& r) override
	{
		const uint32_t *created = nullptr, *lost = nullptr;
		uint32_t nc = 0, nl = 0;
		if(status == GBPX_OK && gbpx_bp_fetch_results(handle, &created, &nc, &lost, &nl) == GBPX_OK)
		{
			r.mNbCreatedPairs = nc;
			r.mCreatedPairs = reinterpret_cast<const PxBroadPhasePair*>(created);
			r.mNbDeletedPairs = nl;
			r.mDeletedPairs = reinterpret_cast<const PxBroadPhasePair*>(lost);
		}
		else
			r = PxBroadPhaseResults();
	}

	PxBroadPhaseDesc desc;
	void* handle;
	int status = GBPX_OK;
	PxAABBManager* manager = nullptr;

private:
	~GbpxBroadPhase() override {}
};

// Per-index bit set (the reference's PxBitMap use: set, reset, test, visit in
// increasing index order).
struct IndexBits
{
	std::vector<uint64_t> words;
	void grow(uint32_t n) { if(words.size() * 64 < n) words.resize((n + 63) / 64, 0); }
	void set(uint32_t i) { grow(i + 1); words[i >> 6] |= 1ull << (i & 63); }
	void reset(uint32_t i) { if((i >> 6) < words.size()) words[i >> 6] &= ~(1ull << (i & 63)); }
	bool test(uint32_t i) const { return (i >> 6) < words.size() && (words[i >> 6] >> (i & 63)) & 1; }
	void clear() { std::fill(words.begin(), words.end(), 0ull); }
	template <typename F> void visit(F f) const
	{
		for(size_t w = 0; w < words.size(); w++)
			for(uint64_t b = words[w]; b; b &= b - 1) f(uint32_t(w * 64 + __builtin_ctzll(b)));
	}
};

constexpr PxBpFilterGroup INVALID_GROUP = 0xffffffffu;   // PX_INVALID_BP_FILTER_GROUP

// The reference's high-level broadphase (NpImmediateMode.cpp:2160-2478): it owns
// bounds / groups / distances arrays (from the broadphase's allocator, grown to
// powers of two, one spare bounds entry for reads past the end), tracks the
// objects added, updated and removed since the last update, and submits them
// in increasing index order.
class GbpxAABBManager : public PxAABBManager
{
public:
	explicit GbpxAABBManager(GbpxBroadPhase& b) : bp(b) { bp.manager = this; }
	void release() override { delete this; }
	PxBroadPhase& getBroadPhase() override { return bp; }
	const PxBounds3* getBounds() const override { return bounds; }
	const float* getDistances() const override { return distances; }
	const PxBpFilterGroup* getGroups() const override { return groups; }
	uint32_t getCapacity() const override { return capacity; }

	void addObject(PxBpIndex index, const PxBounds3& b, PxBpFilterGroup group, float distance) override
	{
		if(capacity < index + 1) reserve(index + 1);
		bounds[index] = b;
		groups[index] = group;
		distances[index] = distance;
		if(removedMap.test(index)) removedMap.reset(index);   // removed and re-added before an update: still in the broadphase
		else addedMap.set(index);
	}
	void removeObject(PxBpIndex index) override
	{
		if(index >= capacity) return;
		if(addedMap.test(index)) addedMap.reset(index);       // added since the last update: never reached the broadphase
		else removedMap.set(index);
		setEmpty(bounds[index]);
		groups[index] = INVALID_GROUP;
		distances[index] = 0.0f;
	}
	void updateObject(PxBpIndex index, const PxBounds3* b, const float* distance) override
	{
		if(index >= capacity) return;
		updatedMap.set(index);
		if(b) bounds[index] = *b;
		if(distance) distances[index] = *distance;
	}
	void update(PxBaseTask* continuation) override
	{
		added.clear();
		updated.clear();
		removed.clear();
		addedMap.visit([&](uint32_t i) { added.push_back(i); });
		updatedMap.visit([&](uint32_t i) { if(!addedMap.test(i)) updated.push_back(i); });   // a new object is not also updated
		removedMap.visit([&](uint32_t i) { removed.push_back(i); });
		const PxBroadPhaseUpdateData data(added.data(), uint32_t(added.size()), updated.data(), uint32_t(updated.size()), removed.data(),
		                                  uint32_t(removed.size()), bounds, groups, distances, capacity);
		bp.update(data, continuation);
		addedMap.clear();
		removedMap.clear();
		updatedMap.clear();
	}
	void fetchResults(PxBroadPhaseResults& r) override { bp.fetchResults(r); }

private:
	~GbpxAABBManager() override
	{
		PxAllocatorCallback* a = bp.getAllocator();
		a->deallocate(distances);
		a->deallocate(groups);
		a->deallocate(bounds);
		bp.manager = nullptr;
	}
	static void setEmpty(PxBounds3& b)   // PxBounds3::setEmpty: inverted maximal bounds
	{
		const float big = 0.25f * 3.402823466e+38f;   // PX_MAX_BOUNDS_EXTENTS
		b.minimum = PxVec3{big, big, big};
		b.maximum = PxVec3{-big, -big, -big};
	}
	void reserve(uint32_t needed)
	{
		uint32_t n = 1;
		while(n < needed) n <<= 1;
		PxAllocatorCallback* a = bp.getAllocator();
		PxBounds3* nb = static_cast<PxBounds3*>(a->allocate(sizeof(PxBounds3) * (n + 1), "bounds", __FILE__, __LINE__));
		PxBpFilterGroup* ng = static_cast<PxBpFilterGroup*>(a->allocate(sizeof(PxBpFilterGroup) * n, "groups", __FILE__, __LINE__));
		float* nd = static_cast<float*>(a->allocate(sizeof(float) * n, "distances", __FILE__, __LINE__));
		if(capacity)
		{
			memcpy(nb, bounds, sizeof(PxBounds3) * capacity);
			memcpy(ng, groups, sizeof(PxBpFilterGroup) * capacity);
			memcpy(nd, distances, sizeof(float) * capacity);
		}
		for(uint32_t i = capacity; i <= n; i++) setEmpty(nb[i]);
		for(uint32_t i = capacity; i < n; i++) { ng[i] = INVALID_GROUP; nd[i] = 0.0f; }
		a->deallocate(bounds);
		a->deallocate(groups);
		a->deallocate(distances);
		bounds = nb;
		groups = ng;
		distances = nd;
		capacity = n;
	}

	GbpxBroadPhase& bp;
	PxBounds3* bounds = nullptr;
	PxBpFilterGroup* groups = nullptr;
	float* distances = nullptr;
	uint32_t capacity = 0;
	IndexBits addedMap, removedMap, updatedMap;
	std::vector<uint32_t> added, updated, removed;
};
} // namespace

GX PxBpFilterGroup PxGetBroadPhaseStaticFilterGroup() { return gbpx_bp_static_filter_group(); }
GX PxBpFilterGroup PxGetBroadPhaseDynamicFilterGroup(uint32_t id) { return gbpx_bp_dynamic_filter_group(id); }
GX PxBpFilterGroup PxGetBroadPhaseKinematicFilterGroup(uint32_t id) { return gbpx_bp_kinematic_filter_group(id); }

GX PxBroadPhase* PxCreateBroadPhase(const PxBroadPhaseDesc& desc)
{
	if(desc.mType != PxBroadPhaseType::eABP && desc.mType != PxBroadPhaseType::ePABP) return nullptr;
	void* h = nullptr;
	if(gbpx_bp_create(desc.mDiscardStaticVsKinematic ? 1 : 0, desc.mDiscardKinematicVsKinematic ? 1 : 0, &h) != GBPX_OK) return nullptr;
	return new GbpxBroadPhase(desc, h);
}

GX PxAABBManager* PxCreateAABBManager(PxBroadPhase& broadphase)
{
	GbpxBroadPhase& bp = static_cast<GbpxBroadPhase&>(broadphase);
	if(bp.manager) return nullptr;   // one manager per broadphase
	return new GbpxAABBManager(bp);
}

// ------------------------------------------------------------------ profiler
// PxSetProfilerCallback (physx/include/foundation/PxFoundation.h:195): the
// library's profiler zones go to the user's PxProfilerCallback.
namespace
{
PxProfilerCallback* gProfiler = nullptr;
void* profZoneStart(const char* name, int detached, uint64_t context, void* user)
{
	return static_cast<PxProfilerCallback*>(user)->zoneStart(name, detached != 0, context);
}
void profZoneEnd(void* data, const char* name, int detached, uint64_t context, void* user)
{
	static_cast<PxProfilerCallback*>(user)->zoneEnd(data, name, detached != 0, context);
}
} // namespace

GX void PxSetProfilerCallback(PxProfilerCallback* profiler)
{
	gProfiler = profiler;
	if(profiler) gbpx_set_profiler_callback(profZoneStart, profZoneEnd, profiler);
	else gbpx_set_profiler_callback(nullptr, nullptr, nullptr);
}

GX PxProfilerCallback* PxGetProfilerCallback() { return gProfiler; }
