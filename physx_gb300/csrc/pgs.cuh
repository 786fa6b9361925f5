// Immediate-mode PGS rigid-body contacts on the device: the solver bodies of
// PxConstructSolverBodies / PxConstructStaticSolverBody
// (physx/source/immediatemode/src/NpImmediateMode.cpp:55,70;
// lowleveldynamics/src/DyRigidBodyToSolverBody.cpp:38), the rows of
// PxCreateContactConstraints (NpImmediateMode.cpp:292) for both of the
// reference's paths — per pair (setupFinalizeSolverConstraints,
// lowleveldynamics/src/DyContactPrep.cpp:49, constructContactConstraint
// DyContactPrepShared.h:298) and the 4-wide block of a header of stride 4
// (setupFinalizeSolverConstraints4, DyContactPrep4.cpp:51) —, the iterations of
// PxSolveConstraints (NpImmediateMode.cpp:552: solveContact / solveContact_BStatic
// DySolverConstraints.cpp:221,373, concludeContact :508; solveContact4_Block /
// solveContact4_StaticBlock / concludeContact4_Block
// DySolverConstraintsBlock.cpp:45,407,676) and PxIntegrateSolverBodies
// (integrateCore, DyBodyCoreIntegrator.h:83).
//
// Every value follows the reference's evaluation order (the translation unit is
// compiled without fused multiply-add).  A lane of a 4-wide header is computed
// alone with the block path's arithmetic: its lanes never exchange values, and
// the padding rows a shorter lane gets carry a zero velocity multiplier.  The
// settings are the immediate-mode snippet's: fresh friction data, unit mass
// scales, zero rest distance and offset slop, no target velocities, unbounded
// maximum impulses, non-negative restitution.
//
// GB300 layout: one 16-byte-aligned record per constraint (its patches, points
// and friction rows with their impulses, 880 bytes at most); a thread prepares
// and solves one record.
#pragma once
#include "solver.cuh"

namespace gbpx
{
namespace pgs
{
using tgs::Contact;
using tgs::Correlation;
using tgs::RigidBody;
using tgs::MAX_CONTACTS;
using tgs::MAX_FRICTION;

// PxSolverBodyData fields the path uses (invMass, penBiasClamp and
// maxContactImpulse in the W lanes)
struct __align__(16) BodyData
{
	V3 lin; float invMass;
	V3 ang; float penBiasClamp;
	M33 sqrtInvInertia; float maxContactImpulse;
	Tr pose;
};
// PxSolverBody: the delta linear velocity and the angular state
struct __align__(16) BodyVel { V3 lin; float pad0; V3 ang; float pad1; };

struct __align__(16) PatchRow
{
	V3 normal;
	float invMass0, invMass1, angDom0, angDom1, staticFriction, dynamicFriction;
	int nbPoints, nbFriction, pad;
};
// conclude: the per-pair path's unbiased error, or the block path's bias
// subtracted at the conclude
struct __align__(16) PointRow { V3 raXn; float velMultiplier; V3 rbXn; float biasedErr; float conclude, impulseMultiplier, force, pad; };
// per-pair rows: bias and target velocity; block rows: the scaled bias and what
// the conclude leaves in it
struct __align__(16) FrictionRow { V3 normal; float appliedForce; V3 raXn; float velMultiplier; V3 rbXn; float bias; float targetVel, pad[3]; };

// flags: REC_BLOCK a lane of a 4-wide header; REC_BLOCK_DYNAMIC that header has
// a dynamic body B; REC_STORE_B the block solve stores body B (its data index is
// not 0); REC_DYNAMIC_B the per-pair solve treats body B as dynamic (the
// header's type is DY_SC_TYPE_RB_CONTACT)
constexpr int REC_BLOCK = 1, REC_BLOCK_DYNAMIC = 2, REC_STORE_B = 4, REC_DYNAMIC_B = 8;
struct __align__(16) Record
{
	int bodyA, bodyB, nbPatches, flags;
	PatchRow patch[MAX_CONTACTS];
	PointRow point[MAX_CONTACTS];
	FrictionRow friction[MAX_FRICTION];
};

// the drop-in reads the point count and the impulses out of a record's bytes
static_assert(sizeof(PatchRow) == 48 && offsetof(PatchRow, nbPoints) == 36, "PatchRow layout");
static_assert(sizeof(PointRow) == 48 && offsetof(PointRow, force) == 40, "PointRow layout");
static_assert(offsetof(Record, patch) == 16 && offsetof(Record, point) == 16 + MAX_CONTACTS * sizeof(PatchRow), "Record layout");

// copyToSolverBodyData (DyRigidBodyToSolverBody.cpp:38) after
// bodyCoreComputeUnconstrainedVelocity (DyBodyCoreIntegrator.h:38)
__device__ __forceinline__ void copyToSolverBody(V3 lv, V3 av, float invMass, V3 invInertia, const Tr& pose, float maxDepen, float maxImpulse,
                                                 BodyData& d)
{
	const M33 rot = m33FromQuatCol(pose.q);   // PxMat33Padded
	const V3 sqrtInv = v3(invInertia.x == 0.0f ? 0.0f : sqrtf(invInertia.x), invInertia.y == 0.0f ? 0.0f : sqrtf(invInertia.y),
	                      invInertia.z == 0.0f ? 0.0f : sqrtf(invInertia.z));
	d.sqrtInvInertia = tgs::transformInertia(sqrtInv, rot);
	d.lin = lv;
	d.ang = av;
	d.invMass = invMass;
	d.penBiasClamp = maxDepen;
	d.maxContactImpulse = maxImpulse;
	d.pose = pose;
}

__device__ __forceinline__ void constructDynamicBody(const RigidBody& r, V3 g, float dt, BodyData& d)
{
	V3 lv = v3(r.linVel[0], r.linVel[1], r.linVel[2]);
	V3 av = v3(r.angVel[0], r.angVel[1], r.angVel[2]);
	// bodyCoreComputeUnconstrainedVelocity
	const float ld = r.linearDamping * dt, ad = r.angularDamping * dt;
	const float oml = 1.0f - ld, oma = 1.0f - ad;
	lv = add(lv, scale(scale(g, dt), 1.0f));
	lv = scale(lv, oml >= 0.0f ? oml : 0.0f);
	av = scale(av, oma >= 0.0f ? oma : 0.0f);
	const float l2 = lenSqS(lv);
	if(l2 > r.maxLinearVelocitySq) lv = scale(lv, sqrtf(r.maxLinearVelocitySq / l2));
	const float a2 = lenSqS(av);
	if(a2 > r.maxAngularVelocitySq) av = scale(av, sqrtf(r.maxAngularVelocitySq / a2));
	Tr pose;
	pose.q.x = r.q[0]; pose.q.y = r.q[1]; pose.q.z = r.q[2]; pose.q.w = r.q[3];
	pose.p = v3(r.p[0], r.p[1], r.p[2]);
	copyToSolverBody(lv, av, r.invMass, v3(r.invInertia[0], r.invInertia[1], r.invInertia[2]), pose, -r.maxDepenetrationVelocity,
	                 r.maxContactImpulse, d);
}

__device__ __forceinline__ void constructStaticBody(const Tr& pose, BodyData& d)
{
	copyToSolverBody(zero3(), zero3(), 0.0f, zero3(), pose, -FLT_MAX, FLT_MAX, d);
}

struct PrepParams { float invDt, bounceThreshold, frictionOffsetThreshold; };

// ------------------------------------------------------------- per-pair rows
__device__ __forceinline__ void prepPair(const Contact* contacts, int nbContacts, int a, int b, const BodyData& d0, const BodyData& d1,
                                         const PrepParams& pp, bool dynamicB, Record& rec)
{
	rec.bodyA = a;
	rec.bodyB = b;
	rec.nbPatches = 0;
	rec.flags = dynamicB ? REC_DYNAMIC_B : 0;
	if(nbContacts == 0) return;
	const Tr& f0 = d0.pose;
	const Tr& f1 = d1.pose;
	Correlation c;
	tgs::getFrictionPatches(c, nullptr, f0, f1, 0.0f);
	tgs::createContactPatches(c, contacts, nbContacts, 0.999f);
	tgs::correlatePatches(c, contacts, f0, f1, 0.999f);
	tgs::growPatches(c, contacts, f0, f1, pp.frictionOffsetThreshold + 0.0f);

	const float invMass0D0 = 1.0f * d0.invMass;
	const float invMass1D1 = (-1.0f) * d1.invMass;   // nDom1 * invMass1
	const float angD0 = 1.0f, angD1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.lin, lv1 = d1.lin, av0 = d0.ang, av1 = d1.ang;
	const float invDt = pp.invDt;
	const float p8 = 0.8f;
	const float invDtp8 = invDt * p8;
	int nPoints = 0, nFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		const int head = c.listHead[i];
		const Contact& base0 = contacts[c.cpStart[head]];
		const float restitution = base0.restitution;
		PatchRow& pr = rec.patch[rec.nbPatches++];
		pr.invMass0 = invMass0D0;
		pr.invMass1 = -invMass1D1;
		pr.angDom0 = angD0; pr.angDom1 = angD1;
		const V3 n = base0.n;
		const float nLenSq = dotA(n, n);
		const float norVel = sumElems(sub(mul(n, lv0), mul(n, lv1)));
		const float imn0 = invMass0D0 * nLenSq, imn1 = invMass1D1 * nLenSq;
		pr.normal = n;
		int pts = 0;
		for(int patch = head; patch != -1; patch = c.cpNext[patch])
			for(int j = 0; j < c.cpCount[patch]; j++)
			{
				const Contact& ct = contacts[c.cpStart[patch] + j];
				const float cTargetVel = dotA(n, zero3());
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				// offsetSlop is 0: the slop test keeps raXn / rbXn as they are
				const float vRelAng = dotA(raXn, av0) - dotA(rbXn, av1);
				const float vrel = norVel + vRelAng;
				const V3 ri0 = m33MulV(d0.sqrtInvInertia, raXn), ri1 = m33MulV(d1.sqrtInvInertia, rbXn);
				const float resp0 = imn0 + dotA(ri0, ri0) * angD0;
				const float resp1 = dotA(ri1, ri1) * angD1 - imn1;
				const float unitResponse = resp0 + resp1;
				const float penetration = ct.sep - 0.0f;
				const float penetrationInvDt = penetration * invDt;
				const bool isSeparated = penetration >= 0.0f;
				const bool collidingWithVrel = -vrel > penetrationInvDt;
				const bool isGreater2 = (restitution > 0.0f && pp.bounceThreshold > vrel) && collidingWithVrel;
				float targetVelocity = cTargetVel + (isGreater2 ? (-vrel) * restitution : 0.0f);
				targetVelocity = targetVelocity - vrel;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				const float velMultiplier = recipResponse;
				const float penetrationInvDtScaled = isSeparated ? penetrationInvDt : penetration * invDtp8;
				float scaledBias = velMultiplier * fmax_(maxPenBias, penetrationInvDtScaled);
				const bool ccdSeparationCondition = FLT_MAX >= penetration;
				scaledBias = (ccdSeparationCondition && isGreater2) ? 0.0f : scaledBias;
				PointRow& row = rec.point[nPoints + pts++];
				row.raXn = ri0;
				row.rbXn = ri1;
				row.velMultiplier = velMultiplier;
				row.impulseMultiplier = 1.0f;
				row.biasedErr = targetVelocity * velMultiplier + (-scaledBias);
				row.conclude = targetVelocity * velMultiplier + (isGreater2 ? 0.0f : -fmax_(scaledBias, 0.0f));
				row.force = 0.0f;
			}
		pr.nbPoints = pts;
		nPoints += pts;
		const int anchors = c.fpAnchorCount[i];
		const float frictionCoefficient = anchors == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * frictionCoefficient;
		pr.dynamicFriction = base0.dynamicFriction * frictionCoefficient;
		pr.nbFriction = anchors * 2;
		if(anchors)
		{
			const V3 linVrel = sub(lv0, lv1);
			const V3 t0f1 = v3(0.0f, -n.z, n.y), t0f2 = v3(-n.y, n.x, 0.0f);
			const V3 t0Fallback = 0.70710678f > fabsf(n.x) ? t0f1 : t0f2;
			V3 t0 = sub(linVrel, scale(n, dotA(n, linVrel)));
			t0 = dotA(t0, t0) > 0.0001f ? t0 : t0Fallback;
			t0 = normalizeA(t0);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < anchors; j++)
			{
				const V3 ra = qRotate(f0.q, c.fpAnchor0[i][j]);
				const V3 rb = qRotate(f1.q, c.fpAnchor1[i][j]);
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					const V3 raXn = cross(ra, t), rbXn = cross(rb, t);
					const V3 ri0 = m33MulV(d0.sqrtInvInertia, raXn), ri1 = m33MulV(d1.sqrtInvInertia, rbXn);
					const float resp0 = invMass0D0 + angD0 * dotA(ri0, ri0);
					const float resp1 = angD1 * dotA(ri1, ri1) - invMass1D1;
					const float resp = resp0 + resp1;
					const float velMultiplier = resp > 0.0f ? p8 / resp : 0.0f;
					float targetVel = dotA(zero3(), t);
					const float vrel1 = dotA(t, lv0) + dotA(raXn, av0);
					const float vrel2 = dotA(t, lv1) + dotA(rbXn, av1);
					targetVel = targetVel - (vrel1 - vrel2);
					FrictionRow& fr = rec.friction[nFriction++];
					fr.normal = t;
					fr.appliedForce = 0.0f;
					fr.raXn = ri0;
					fr.velMultiplier = velMultiplier;
					fr.rbXn = ri1;
					fr.bias = dotA(t, error) * invDt;
					fr.targetVel = targetVel;
				}
			}
		}
	}
}

// ------------------------------------------------------------- one lane of a 4-wide block
__device__ __forceinline__ void prepBlockLane(const Contact* contacts, int nbContacts, int a, int b, const BodyData& d0, const BodyData& d1,
                                              const PrepParams& pp, bool blockDynamic, bool storeB, Record& rec)
{
	rec.bodyA = a;
	rec.bodyB = b;
	rec.nbPatches = 0;
	rec.flags = REC_BLOCK | (blockDynamic ? REC_BLOCK_DYNAMIC : 0) | (storeB ? REC_STORE_B : 0);
	if(nbContacts == 0) return;
	const Tr& f0 = d0.pose;
	const Tr& f1 = d1.pose;
	Correlation c;
	tgs::getFrictionPatches(c, nullptr, f0, f1, 0.0f);
	tgs::createContactPatches(c, contacts, nbContacts, 0.999f);
	tgs::correlatePatches(c, contacts, f0, f1, 0.999f);
	tgs::growPatches(c, contacts, f0, f1, pp.frictionOffsetThreshold + 0.0f);

	const float angDom0 = 1.0f, angDom1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 lv0 = d0.lin, lv1 = d1.lin, av0 = d0.ang, av1 = d1.ang;
	const float invMass0D0 = 1.0f * d0.invMass, invMass1D1 = 1.0f * d1.invMass;
	const M33& I0 = d0.sqrtInvInertia;
	const M33& I1 = d1.sqrtInvInertia;
	const V3 p0 = f0.p, p1 = f1.p;
	const float invDt = pp.invDt;
	const float p8 = 0.8f;
	const float invDtp8 = invDt * p8;
	const V3 vrelv = sub(lv0, lv1);
	int nPoints = 0, nFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		const int head = c.listHead[i];
		const Contact& base0 = contacts[c.cpStart[head]];
		const float restitution = -base0.restitution;
		PatchRow& pr = rec.patch[rec.nbPatches++];
		pr.invMass0 = invMass0D0;
		pr.invMass1 = invMass1D1;
		pr.angDom0 = angDom0; pr.angDom1 = angDom1;
		const V3 n = base0.n;
		pr.normal = n;
		const float relNorVel = tgs::dotXYZ(n, lv0) - tgs::dotXYZ(n, lv1);
		int pts = 0;
		for(int patch = head; patch != -1; patch = c.cpNext[patch])
			for(int j = 0; j < c.cpCount[patch]; j++)
			{
				const Contact& ct = contacts[c.cpStart[patch] + j];
				const float cTargetNorVel = tgs::dotZYX(zero3(), n);
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				const float relAng = tgs::dotXYZ(raXn, av0) - tgs::dotXYZ(rbXn, av1);
				const V3 delAng0 = tgs::m33TMulXYZ(I0, raXn);
				float unitResponse = tgs::dotZYX(delAng0, delAng0) * angDom0 + invMass0D0;
				const float vrel = relNorVel + relAng;
				V3 delAng1 = zero3();
				if(blockDynamic)
				{
					delAng1 = tgs::m33TMulXYZ(I1, rbXn);
					const float resp1 = tgs::dotZYX(delAng1, delAng1) * angDom1 + invMass1D1;
					unitResponse = unitResponse + resp1;
				}
				const float penetration = ct.sep - 0.0f;
				const float penInvDtPt8 = fmax_(maxPenBias, penetration * invDtp8);
				const float penetrationInvDt = penetration * invDt;
				const bool isSeparated = penetration >= 0.0f;
				const bool collidingWithVrel = -vrel > penetrationInvDt;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				const float velMultiplier = recipResponse;   // restitution >= 0: not compliant
				float scaledBias = (isSeparated ? penetrationInvDt : penInvDtPt8) * velMultiplier;
				const bool isGreater2 = (0.0f > restitution && pp.bounceThreshold > vrel) && collidingWithVrel;
				const bool ccdSeparationCondition = FLT_MAX >= penetration;
				scaledBias = -((ccdSeparationCondition && isGreater2) ? 0.0f : scaledBias);
				const float targetVelocity = ((cTargetNorVel - vrel) + (isGreater2 ? vrel * restitution : 0.0f)) * velMultiplier;
				PointRow& row = rec.point[nPoints + pts++];
				row.raXn = delAng0;
				row.rbXn = delAng1;
				row.velMultiplier = velMultiplier;
				row.biasedErr = targetVelocity + scaledBias;
				row.impulseMultiplier = 1.0f - 0.0f;
				row.conclude = isGreater2 ? scaledBias : fmax_(0.0f, scaledBias);
				row.force = 0.0f;
			}
		pr.nbPoints = pts;
		nPoints += pts;
		const int anchors = c.fpAnchorCount[i];
		const float coefficient = anchors == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * coefficient;
		pr.dynamicFriction = base0.dynamicFriction * coefficient;
		pr.nbFriction = anchors * 2;
		if(anchors)
		{
			const V3 fb1 = v3(0.0f, -n.z, n.y), fb2 = v3(-n.y, n.x, 0.0f);
			const V3 fallback = 0.70710678f > fabsf(n.x) ? fb1 : fb2;
			const V3 vs = v3(vrelv.x - n.x * relNorVel, vrelv.y - n.y * relNorVel, vrelv.z - n.z * relNorVel);
			V3 t0 = tgs::dotZYX(vs, vs) > 0.0001f ? vs : fallback;
			const float recipLen = 1.0f / sqrtf(tgs::dotXYZ(t0, t0));
			t0 = scale(t0, recipLen);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < anchors; j++)
			{
				const V3 ra = tgs::qRotate4V(f0.q, c.fpAnchor0[i][j]);
				const V3 rb = tgs::qRotate4V(f1.q, c.fpAnchor1[i][j]);
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					const V3 raXn = cross(ra, t);
					const V3 delAng0 = tgs::m33TMulXYZ(I0, raXn);
					// the friction rows sum their squares z + (y + x), the normal rows x + (y + z)
					float resp = tgs::dotXYZ(delAng0, delAng0) * angDom0 + invMass0D0;
					const float tVel0 = tgs::dotXYZ(t, lv0);
					float vrel = ((tVel0 + raXn.x * av0.x) + raXn.y * av0.y) + raXn.z * av0.z;
					V3 delAng1 = zero3();
					if(blockDynamic)
					{
						const V3 rbXn = cross(rb, t);
						delAng1 = tgs::m33TMulXYZ(I1, rbXn);
						const float resp1 = tgs::dotXYZ(delAng1, delAng1) * angDom1 + invMass1D1;
						resp = resp + resp1;
						const float tVel1 = tgs::dotXYZ(t, lv1);
						const float vel1 = ((tVel1 + rbXn.x * av1.x) + rbXn.y * av1.y) + rbXn.z * av1.z;
						vrel = vrel - vel1;
					}
					const float velMultiplier = 1.0f * (resp > 0.0f ? p8 / resp : 0.0f);
					float bias = tgs::dotXYZ(t, error) * invDt;
					const float targetVel = tgs::dotXYZ(t, zero3()) - vrel;
					FrictionRow& fr = rec.friction[nFriction++];
					fr.normal = t;
					fr.raXn = delAng0;
					fr.rbXn = delAng1;
					fr.appliedForce = 0.0f;
					fr.velMultiplier = velMultiplier;
					fr.targetVel = -(targetVel * velMultiplier);
					bias = bias - targetVel;
					fr.bias = bias * velMultiplier;
				}
			}
		}
	}
}

// ------------------------------------------------------------- solve
// solveContact (dynamic body B) / solveContact_BStatic, then concludeContact
__device__ __forceinline__ void solvePair(Record& rec, BodyVel& b0, BodyVel& b1, bool doFriction, bool conclude)
{
	const bool dynamicB = (rec.flags & REC_DYNAMIC_B) != 0;
	V3 linVel0 = b0.lin, angState0 = b0.ang, linVel1 = b1.lin, angState1 = b1.ang;
	int pointBase = 0, frictionBase = 0;
	for(int k = 0; k < rec.nbPatches; k++)
	{
		const PatchRow& pr = rec.patch[k];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1, angDom0 = pr.angDom0, angDom1 = pr.angDom1;
		float accumulated = 0.0f;
		const V3 delLinVel0 = scale(n, invMassA);
		const V3 delLinVel1 = scale(n, invMassB);
		for(int i = 0; i < pr.nbPoints; i++)
		{
			PointRow& c = rec.point[pointBase + i];
			const float appliedForce = c.force;
			float normalVel;
			if(dynamicB)
				normalVel = sumElems(sub(add(mul(linVel0, n), mul(angState0, c.raXn)), add(mul(linVel1, n), mul(angState1, c.rbXn))));
			else
				normalVel = sumElems(add(mul(linVel0, n), mul(angState0, c.raXn)));
			const float _deltaF = fmax_(c.biasedErr - normalVel * c.velMultiplier, -appliedForce);
			const float _newForce = c.impulseMultiplier * appliedForce + _deltaF;
			const float newForce = fmin_(_newForce, FLT_MAX);
			const float deltaF = newForce - appliedForce;
			linVel0 = add(scale(delLinVel0, deltaF), linVel0);
			angState0 = add(scale(c.raXn, deltaF * angDom0), angState0);
			if(dynamicB)
			{
				linVel1 = sub(linVel1, scale(delLinVel1, deltaF));
				angState1 = sub(angState1, scale(c.rbXn, deltaF * angDom1));
			}
			c.force = newForce;
			accumulated = accumulated + newForce;
		}
		if(doFriction && pr.nbFriction)
		{
			const float maxFrictionImpulse = pr.staticFriction * accumulated;
			const float maxDynFrictionImpulse = pr.dynamicFriction * accumulated;
			const float negMaxDynFrictionImpulse = -maxDynFrictionImpulse;
			for(int i = 0; i < pr.nbFriction; i++)
			{
				FrictionRow& f = rec.friction[frictionBase + i];
				const V3 t = f.normal;
				const float appliedForce = f.appliedForce;
				float normalVel;
				if(dynamicB)
					normalVel = sumElems(sub(add(mul(linVel0, t), mul(angState0, f.raXn)), add(mul(linVel1, t), mul(angState1, f.rbXn))));
				else
					normalVel = sumElems(add(mul(linVel0, t), mul(angState0, f.raXn)));
				const float tmp1 = appliedForce - (f.bias - f.targetVel) * f.velMultiplier;
				const float totalImpulse = tmp1 - normalVel * f.velMultiplier;
				const bool clamp = fabsf(totalImpulse) > maxFrictionImpulse;
				const float totalClamped = fmin_(maxDynFrictionImpulse, fmax_(negMaxDynFrictionImpulse, totalImpulse));
				const float newAppliedForce = clamp ? totalClamped : totalImpulse;
				const float deltaF = newAppliedForce - appliedForce;
				linVel0 = add(scale(scale(t, invMassA), deltaF), linVel0);
				angState0 = add(scale(f.raXn, deltaF * angDom0), angState0);
				if(dynamicB)
				{
					linVel1 = sub(linVel1, scale(scale(t, invMassB), deltaF));
					angState1 = sub(angState1, scale(f.rbXn, deltaF * angDom1));
				}
				f.appliedForce = newAppliedForce;
			}
		}
		if(conclude)
		{
			for(int i = 0; i < pr.nbPoints; i++) rec.point[pointBase + i].biasedErr = rec.point[pointBase + i].conclude;
			for(int i = 0; i < pr.nbFriction; i++) rec.friction[frictionBase + i].bias = 0.0f;
		}
		pointBase += pr.nbPoints;
		frictionBase += pr.nbFriction;
	}
	b0.lin = linVel0;
	b0.ang = angState0;
	b1.lin = linVel1;
	b1.ang = angState1;
}

// one lane of solveContact4_Block / solveContact4_StaticBlock, then concludeContact4_Block
__device__ __forceinline__ void solveBlockLane(Record& rec, BodyVel& b0, BodyVel& b1, bool doFriction, bool conclude)
{
	const bool dynamicBlock = (rec.flags & REC_BLOCK_DYNAMIC) != 0;
	V3 lin0 = b0.lin, ang0 = b0.ang, lin1 = b1.lin, ang1 = b1.ang;
	int pointBase = 0, frictionBase = 0;
	for(int k = 0; k < rec.nbPatches; k++)
	{
		const PatchRow& pr = rec.patch[k];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1, angD0 = pr.angDom0, angD1 = pr.angDom1;
		float accumulated = 0.0f, accumDeltaF = 0.0f;
		if(dynamicBlock)
		{
			const float sumInvMass = invMassA + invMassB;
			float relVel1 = tgs::dotXYZ(lin0, n) - tgs::dotXYZ(lin1, n);
			for(int i = 0; i < pr.nbPoints; i++)
			{
				PointRow& c = rec.point[pointBase + i];
				const float appliedForce = c.force;
				const float normalVel = relVel1 + (tgs::dotXYZ(c.raXn, ang0) - tgs::dotXYZ(c.rbXn, ang1));
				float deltaF = c.biasedErr - normalVel * c.velMultiplier;
				deltaF = fmax_(deltaF, -appliedForce);
				const float newApplied = fmin_(c.impulseMultiplier * appliedForce + deltaF, FLT_MAX);
				deltaF = newApplied - appliedForce;
				accumDeltaF = accumDeltaF + deltaF;
				const float angDeltaF0 = deltaF * angD0, angDeltaF1 = deltaF * angD1;
				relVel1 = sumInvMass * deltaF + relVel1;
				ang0 = add(scale(c.raXn, angDeltaF0), ang0);
				ang1 = sub(ang1, scale(c.rbXn, angDeltaF1));
				c.force = newApplied;
				accumulated = accumulated + newApplied;
			}
			lin0 = add(scale(n, accumDeltaF * invMassA), lin0);
			lin1 = sub(lin1, scale(n, accumDeltaF * invMassB));
		}
		else
		{
			float cnv1 = tgs::dotXYZ(lin0, n);
			for(int i = 0; i < pr.nbPoints; i++)
			{
				PointRow& c = rec.point[pointBase + i];
				const float appliedForce = c.force;
				const float normalVel = ((cnv1 + c.raXn.x * ang0.x) + c.raXn.y * ang0.y) + c.raXn.z * ang0.z;
				const float _deltaF = fmax_(c.biasedErr - normalVel * c.velMultiplier, -appliedForce);
				const float newApplied = fmin_(c.impulseMultiplier * appliedForce + _deltaF, FLT_MAX);
				const float deltaF = newApplied - appliedForce;
				accumDeltaF = accumDeltaF + deltaF;
				cnv1 = invMassA * deltaF + cnv1;
				ang0 = add(scale(c.raXn, angD0 * deltaF), ang0);
				c.force = newApplied;
				accumulated = accumulated + newApplied;
			}
			lin0 = add(scale(n, accumDeltaF * invMassA), lin0);
		}
		if(doFriction && pr.nbFriction)
		{
			const float maxFrictionImpulse = pr.staticFriction * accumulated;
			const float maxDynFrictionImpulse = pr.dynamicFriction * accumulated;
			const float negMaxDynFrictionImpulse = -maxDynFrictionImpulse;
			bool broken = false;
			for(int i = 0; i < pr.nbFriction; i++)
			{
				FrictionRow& f = rec.friction[frictionBase + i];
				const V3 t = f.normal;
				const float appliedForce = f.appliedForce;
				const float normalVel = dynamicBlock
				                            ? (tgs::dotXYZ(lin0, t) + tgs::dotXYZ(f.raXn, ang0)) - (tgs::dotXYZ(lin1, t) + tgs::dotXYZ(f.rbXn, ang1))
				                            : tgs::dotXYZ(lin0, t) + tgs::dotXYZ(f.raXn, ang0);
				const float tmp1 = appliedForce - f.bias;
				const float totalImpulse = tmp1 - normalVel * f.velMultiplier;
				broken = broken || fabsf(totalImpulse) > maxFrictionImpulse;   // carried across the patch's rows
				const float newApplied = broken ? fmin_(maxDynFrictionImpulse, fmax_(negMaxDynFrictionImpulse, totalImpulse)) : totalImpulse;
				const float deltaF = newApplied - appliedForce;
				f.appliedForce = newApplied;
				if(dynamicBlock)
				{
					lin0 = add(scale(t, deltaF * invMassA), lin0);
					lin1 = sub(lin1, scale(t, deltaF * invMassB));
					ang0 = add(scale(f.raXn, deltaF * angD0), ang0);
					ang1 = sub(ang1, scale(f.rbXn, deltaF * angD1));
				}
				else
				{
					lin0 = add(scale(t, invMassA * deltaF), lin0);
					ang0 = add(scale(f.raXn, angD0 * deltaF), ang0);
				}
			}
		}
		if(conclude)
		{
			for(int i = 0; i < pr.nbPoints; i++) rec.point[pointBase + i].biasedErr = rec.point[pointBase + i].biasedErr - rec.point[pointBase + i].conclude;
			for(int i = 0; i < pr.nbFriction; i++) rec.friction[frictionBase + i].bias = rec.friction[frictionBase + i].targetVel;
		}
		pointBase += pr.nbPoints;
		frictionBase += pr.nbFriction;
	}
	b0.lin = lin0;
	b0.ang = ang0;
	b1.lin = lin1;
	b1.ang = ang1;
}

// integrateCore (DyBodyCoreIntegrator.h:83): the motion velocities of the
// position iterations move the pose, the solver deltas update the velocities.
// sin/cos are evaluated in double and rounded: the host C library's sinf/cosf
// that the reference calls are nearer to the correctly rounded values than the
// device's single-precision functions.
__device__ __forceinline__ void integrateBody(V3 motionLin, V3 motionAng, const BodyVel& sb, BodyData& d, float dt)
{
	const V3 linearMotionVel = add(d.lin, motionLin);
	d.pose.p = add(d.pose.p, scale(linearMotionVel, dt));
	V3 angularMotionVel = add(d.ang, m33MulVS(d.sqrtInvInertia, motionAng));
	float w = lenSqS(angularMotionVel);
	if(w != 0.0f)
	{
		w = sqrtf(w);
		const float maxW = 1e+7f;
		if(w > maxW)
		{
			angularMotionVel = scale(normalizeS(angularMotionVel), maxW);
			w = maxW;
		}
		const float v = dt * w * 0.5f;
		float s, q;
		sinCosAngle(v, s, q);   // correctly rounded (the host C library's sinf / cosf match it far more often than the device ones)
		s = s / w;
		const V3 pqr = scale(angularMotionVel, s);
		const Q quatVel = {pqr.x, pqr.y, pqr.z, 0.0f};
		Q result = qMulS(quatVel, d.pose.q);
		const Q q0 = d.pose.q;
		result.x += q0.x * q; result.y += q0.y * q; result.z += q0.z * q; result.w += q0.w * q;
		const float m = sqrtf(result.x * result.x + result.y * result.y + result.z * result.z + result.w * result.w);
		const float r = 1.0f / m;
		d.pose.q.x = result.x * r; d.pose.q.y = result.y * r; d.pose.q.z = result.z * r; d.pose.q.w = result.w * r;
	}
	d.lin = add(d.lin, sb.lin);
	d.ang = add(d.ang, m33MulVS(d.sqrtInvInertia, sb.ang));
}
} // namespace pgs
} // namespace gbpx
