// TGS contact solver building blocks for the GB300 rigid-body step.
//
// Follows the reference's immediate-mode TGS contact path:
//   body construction: bodyCoreComputeUnconstrainedVelocity
//     (physx/source/lowleveldynamics/src/DyBodyCoreIntegrator.h:38) and
//     copyToSolverBodyDataStep (DyTGSDynamics.cpp:154);
//   batching: classifyConstraintDesc / writeConstraintDesc
//     (DyConstraintPartition.cpp:476,571) and createHeaders
//     (physx/source/immediatemode/src/NpImmediateMode.cpp:159);
//   rows: createContactPatches / correlatePatches / growPatches
//     (DyFrictionCorrelation.cpp:56,133,187), setupFinalizeSolverConstraints
//     and constructContactConstraintStep (DyTGSContactPrep.cpp:426,322);
//   solve: solveContact / solveDynamicContactsStep (DyTGSContactPrep.cpp:1581,1492);
//   integration: integrateCoreStep (DyTGSDynamics.cpp:1403) and
//     PxIntegrateSolverBodiesTGS (NpImmediateMode.cpp:1719).
// Settings are those of immediate-mode callers: friction patches fresh or
// carried from the last frame (correlated and grown), unit mass scales, zero
// rest distance and offset slop, no torsional friction.
//
// GB300 layout: a pair has at most 4 contacts, so a constraint's rows fit a
// record of at most 896 bytes (<= 4 patches, <= 4 point rows, <= 8 friction
// rows), packed to the rows it uses, that the prep pass writes once and every
// solve iteration reads; the
// partitioning (batching) rule guarantees that the constraints of one
// partition touch disjoint dynamic bodies, so a partition is solved as one
// parallel wave and reproduces the reference's sequential order.
#pragma once
#include "vmath.cuh"

namespace gbpx
{
namespace tgs
{
constexpr int MAX_CONTACTS = 4;
constexpr int MAX_FRICTION = 8;

struct RigidBody   // PxRigidBodyData (physx/include/PxImmediateMode.h:68), 96 bytes
{
	float linVel[3]; float invMass;
	float angVel[3]; float maxDepenetrationVelocity;
	float invInertia[3]; float maxContactImpulse;
	float q[4]; float p[3];
	float linearDamping, angularDamping, maxLinearVelocitySq, maxAngularVelocitySq;
	uint32_t pad;
};
static_assert(sizeof(RigidBody) == 96, "PxRigidBodyData layout");

// Solver-body records, 16-byte aligned (64 / 64 / 48 bytes) so that a record spans
// whole 32-byte sectors: every constraint reads two of each.
struct __align__(16) BodyVel { V3 lin, ang, dLin, dAng; float maxAngVel; int kinematic; };      // PxTGSSolverBodyVel fields
struct __align__(16) BodyTx { Q dq; V3 p; M33 sqrtInvInertia; };                                 // PxTGSSolverBodyTxInertia
struct __align__(16) BodyData { V3 origLin, origAng; float maxContactImpulse, penBiasClamp, invMass; };  // PxTGSSolverBodyData

struct Contact { V3 n; float sep; V3 p; float staticFriction, dynamicFriction, restitution; };

struct __align__(16) PointRow { V3 raXnI, rbXnI; float velMultiplier, separation, biasCoefficient, targetVelocity, recipResponse, maxImpulse; };
struct FrictionRow { V3 normal; float error; V3 raXnI; float targetVel; V3 rbXnI; float velMultiplier, frictionScale, biasScale; };
struct __align__(16) PatchRows
{
	V3 normal;
	float invMass0, invMass1, maxPenBias, staticFriction, dynamicFriction;
	int pointStart, nbPoints, frictionStart, nbFriction;
};
// One constraint's rows, packed after a 16-byte header so that a constraint
// touches as few cache lines as it has rows: patches, points, friction rows
// (two per anchor), normal impulses, friction impulses.
// Flags in the high byte of ConstraintRecord::counts.  REC_BLOCK: the rows were
// built, and are solved, by the 4-wide block path (one lane of a header of
// stride 4).  REC_KEEP_B: the block solve leaves body B's velocity as it was
// (the reference stores body B only when its data index is not 0).
constexpr int REC_BLOCK = 1 << 24;
constexpr int REC_KEEP_B = 1 << 25;
struct __align__(16) ConstraintRecord
{
	int bodyA, bodyB, nbPatches, counts;   // counts = points | friction rows << 16 | flags
	float4 rows[(MAX_CONTACTS * sizeof(PatchRows) + MAX_CONTACTS * sizeof(PointRow) + MAX_FRICTION * sizeof(FrictionRow) +
	             (MAX_CONTACTS + MAX_FRICTION) * 4 + 15) / 16];

	__device__ __forceinline__ int nbPoints() const { return counts & 0xffff; }
	__device__ __forceinline__ int nbFriction() const { return (counts >> 16) & 0xff; }
	__device__ __forceinline__ bool isBlock() const { return (counts & REC_BLOCK) != 0; }
	__device__ __forceinline__ bool keepB() const { return (counts & REC_KEEP_B) != 0; }
	__device__ __forceinline__ PatchRows* patch() { return reinterpret_cast<PatchRows*>(rows); }
	__device__ __forceinline__ PointRow* point() { return reinterpret_cast<PointRow*>(reinterpret_cast<char*>(rows) + nbPatches * sizeof(PatchRows)); }
	__device__ __forceinline__ FrictionRow* friction()
	{
		return reinterpret_cast<FrictionRow*>(reinterpret_cast<char*>(point()) + nbPoints() * sizeof(PointRow));
	}
	__device__ __forceinline__ float* force() { return reinterpret_cast<float*>(friction() + nbFriction()); }
	__device__ __forceinline__ float* frictionForce() { return force() + nbPoints(); }
	// bytes the header and packed rows occupy
	__device__ __forceinline__ uint32_t bytes() const
	{
		return 16u + uint32_t(nbPatches) * uint32_t(sizeof(PatchRows)) + uint32_t(nbPoints()) * uint32_t(sizeof(PointRow) + 4) +
		       uint32_t(nbFriction()) * uint32_t(sizeof(FrictionRow) + 4);
	}
};

// ------------------------------------------------------------- bodies
__host__ __device__ __forceinline__ float selPos(float x) { return x >= 0.0f ? x : 0.0f; }

__device__ __forceinline__ M33 transformInertia(V3 d, const M33& M)
{
	// Cm::transformInertiaTensor (physx/source/common/src/CmUtils.h:57), M(r, c) = column c row r
	const float m00 = M.c0.x, m10 = M.c0.y, m20 = M.c0.z;
	const float m01 = M.c1.x, m11 = M.c1.y, m21 = M.c1.z;
	const float m02 = M.c2.x, m12 = M.c2.y, m22 = M.c2.z;
	const float axx = d.x * m00, axy = d.x * m10, axz = d.x * m20;
	const float byx = d.y * m01, byy = d.y * m11, byz = d.y * m21;
	const float czx = d.z * m02, czy = d.z * m12, czz = d.z * m22;
	const float i00 = axx * m00 + byx * m01 + czx * m02;
	const float i11 = axy * m10 + byy * m11 + czy * m12;
	const float i22 = axz * m20 + byz * m21 + czz * m22;
	const float i01 = axx * m10 + byx * m11 + czx * m12;
	const float i02 = axx * m20 + byx * m21 + czx * m22;
	const float i12 = axy * m20 + byy * m21 + czy * m22;
	M33 r;
	r.c0 = v3(i00, i01, i02);
	r.c1 = v3(i01, i11, i12);
	r.c2 = v3(i02, i12, i22);
	return r;
}

__device__ __forceinline__ void copyToSolverBody(V3 lv, V3 av, float invMass, V3 invInertia, const Tr& pose, float maxDepen, float maxImpulse,
                                                 float maxAngVelSq, bool kinematic, BodyVel& vel, BodyTx& tx, BodyData& data)
{
	const M33 rot = m33FromQuatCol(pose.q);   // PxMat33Padded
	const V3 sqrtInv = v3(invInertia.x == 0.0f ? 0.0f : sqrtf(invInertia.x), invInertia.y == 0.0f ? 0.0f : sqrtf(invInertia.y),
	                      invInertia.z == 0.0f ? 0.0f : sqrtf(invInertia.z));
	const V3 sqrtBody = v3(sqrtInv.x == 0.0f ? 0.0f : 1.0f / sqrtInv.x, sqrtInv.y == 0.0f ? 0.0f : 1.0f / sqrtInv.y,
	                       sqrtInv.z == 0.0f ? 0.0f : 1.0f / sqrtInv.z);
	tx.sqrtInvInertia = transformInertia(sqrtInv, rot);
	tx.p = pose.p;
	tx.dq.x = tx.dq.y = tx.dq.z = 0.0f;
	tx.dq.w = 1.0f;
	const M33 sqrtInertia = transformInertia(sqrtBody, rot);
	vel.lin = lv;
	vel.ang = m33MulVS(sqrtInertia, av);
	vel.dLin = zero3();
	vel.dAng = zero3();
	vel.kinematic = kinematic ? 1 : 0;
	vel.maxAngVel = sqrtf(maxAngVelSq);
	data.invMass = invMass;
	data.penBiasClamp = maxDepen;
	data.maxContactImpulse = maxImpulse;
	data.origLin = lv;
	data.origAng = av;
}

// PxConstructSolverBodiesTGS for one body (gravity*dt, damping, clamps, solver body)
__device__ __forceinline__ void constructDynamicBody(const RigidBody& r, V3 g, float dt, BodyVel& vel, BodyTx& tx, BodyData& data, Tr& pose)
{
	V3 lv = v3(r.linVel[0], r.linVel[1], r.linVel[2]);
	V3 av = v3(r.angVel[0], r.angVel[1], r.angVel[2]);
	const float oml = 1.0f - r.linearDamping * dt, oma = 1.0f - r.angularDamping * dt;
	lv = add(lv, scale(scale(g, dt), 1.0f));
	lv = scale(lv, selPos(oml));
	av = scale(av, selPos(oma));
	const float l2 = lenSqS(lv);
	if(l2 > r.maxLinearVelocitySq) lv = scale(lv, sqrtf(r.maxLinearVelocitySq / l2));
	const float a2 = lenSqS(av);
	if(a2 > r.maxAngularVelocitySq) av = scale(av, sqrtf(r.maxAngularVelocitySq / a2));
	pose.q.x = r.q[0]; pose.q.y = r.q[1]; pose.q.z = r.q[2]; pose.q.w = r.q[3];
	pose.p = v3(r.p[0], r.p[1], r.p[2]);
	copyToSolverBody(lv, av, r.invMass, v3(r.invInertia[0], r.invInertia[1], r.invInertia[2]), pose, -r.maxDepenetrationVelocity,
	                 r.maxContactImpulse, r.maxAngularVelocitySq, false, vel, tx, data);
}

// PxConstructStaticSolverBodyTGS (statics are flagged kinematic by the reference)
__device__ __forceinline__ void constructStaticBody(const Tr& pose, BodyVel& vel, BodyTx& tx, BodyData& data)
{
	copyToSolverBody(zero3(), zero3(), 0.0f, zero3(), pose, -FLT_MAX, FLT_MAX, FLT_MAX, true, vel, tx, data);
}

// ------------------------------------------------------------- persistent friction patches
// FrictionPatch (lowleveldynamics/src/DyFrictionPatch.h:43): what a contact
// constraint leaves for the next frame (frictionPtr / frictionCount) and
// reads back then.  A pair of <= 4 contacts writes <= 4 patches.
struct __align__(16) FrictionPatchDev
{
	V3 body0Normal; int broken;
	V3 body1Normal; int anchorCount;
	V3 body0Anchors[2];
	V3 body1Anchors[2];
	float staticFriction, dynamicFriction, restitution, pad;
	Q relativeQuat;
};
static_assert(sizeof(FrictionPatchDev) == 112, "friction patch layout");
struct __align__(16) FrictionState
{
	uint32_t count, pad[3];
	FrictionPatchDev patches[MAX_CONTACTS];
};

// ------------------------------------------------------------- friction correlation (<= 4 contacts, <= 4 kept patches)
constexpr int MAX_FPATCH = 2 * MAX_CONTACTS;   // last frame's patches, then this frame's
struct Correlation
{
	int cpStart[MAX_CONTACTS], cpCount[MAX_CONTACTS], cpNext[MAX_CONTACTS];
	float cpRest[MAX_CONTACTS], cpSF[MAX_CONTACTS], cpDF[MAX_CONTACTS];
	V3 cpMin[MAX_CONTACTS], cpMax[MAX_CONTACTS];
	int contactPatchCount;
	V3 fpWorldNormal[MAX_FPATCH];
	V3 fpAnchor0[MAX_FPATCH][2], fpAnchor1[MAX_FPATCH][2];
	int fpAnchorCount[MAX_FPATCH];
	float fpRest[MAX_FPATCH], fpSF[MAX_FPATCH], fpDF[MAX_FPATCH];
	int fpContactCount[MAX_FPATCH];
	V3 fpMin[MAX_FPATCH], fpMax[MAX_FPATCH];
	int listHead[MAX_FPATCH];
	V3 fpN0[MAX_FPATCH], fpN1[MAX_FPATCH];   // body0Normal, body1Normal
	Q fpQ[MAX_FPATCH];                       // relativeQuat
	int fpBroken[MAX_FPATCH];
	int frictionPatchCount;

	__device__ void exportPatch(int i, FrictionPatchDev& o) const
	{
		o.body0Normal = fpN0[i]; o.body1Normal = fpN1[i];
		o.broken = fpBroken[i]; o.anchorCount = fpAnchorCount[i];
		o.body0Anchors[0] = fpAnchor0[i][0]; o.body0Anchors[1] = fpAnchor0[i][1];
		o.body1Anchors[0] = fpAnchor1[i][0]; o.body1Anchors[1] = fpAnchor1[i][1];
		o.staticFriction = fpSF[i]; o.dynamicFriction = fpDF[i]; o.restitution = fpRest[i]; o.pad = 0.0f;
		o.relativeQuat = fpQ[i];
	}
};

// getFrictionPatches (lowleveldynamics/src/DyContactPrepShared.h:73): last
// frame's patches that are not broken, have anchors, still face each other and
// whose anchors have not separated along the normal by the correlation
// distance start the list, without contacts.
__device__ __forceinline__ void getFrictionPatches(Correlation& c, const FrictionState* prev, const Tr& f0, const Tr& f1, float correlationDistance)
{
	c.frictionPatchCount = 0;
	if(!prev) return;
	const uint32_t count = prev->count < uint32_t(MAX_CONTACTS) ? prev->count : uint32_t(MAX_CONTACTS);
	if(!count) return;
	const Q qinv = qConj(f0.q);
	const V3 b1to0p = qRotateS(qinv, sub(f1.p, f0.p));
	const Q b1to0q = qMulS(qinv, f1.q);
	for(uint32_t k = 0; k < count; k++)
	{
		const FrictionPatchDev patch = prev->patches[k];
		if(patch.broken || patch.anchorCount == 0) continue;
		if(!(dotS(patch.body0Normal, qRotateS(b1to0q, patch.body1Normal)) > 0.999f)) continue;
		bool separated = false;
		for(int a = 0; a < patch.anchorCount; a++)
		{
			const V3 p1in0 = add(qRotateS(b1to0q, patch.body1Anchors[a]), b1to0p);
			if(!(fabsf(dotS(sub(patch.body0Anchors[a], p1in0), patch.body0Normal)) < correlationDistance)) { separated = true; break; }
		}
		if(separated) continue;
		const int i = c.frictionPatchCount++;
		c.fpWorldNormal[i] = qRotateS(f0.q, patch.body0Normal);
		c.fpContactCount[i] = 0;
		c.fpMin[i] = v3(FLT_MAX, FLT_MAX, FLT_MAX);
		c.fpMax[i] = v3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
		c.listHead[i] = -1;
		c.fpN0[i] = patch.body0Normal; c.fpN1[i] = patch.body1Normal;
		c.fpBroken[i] = patch.broken; c.fpAnchorCount[i] = patch.anchorCount;
		c.fpAnchor0[i][0] = patch.body0Anchors[0]; c.fpAnchor0[i][1] = patch.body0Anchors[1];
		c.fpAnchor1[i][0] = patch.body1Anchors[0]; c.fpAnchor1[i][1] = patch.body1Anchors[1];
		c.fpSF[i] = patch.staticFriction; c.fpDF[i] = patch.dynamicFriction; c.fpRest[i] = patch.restitution;
		c.fpQ[i] = patch.relativeQuat;
	}
}

__device__ __forceinline__ void createContactPatches(Correlation& c, const Contact* cb, int n, float tol)
{
	c.contactPatchCount = 0;
	if(!n) return;
	int pc = 0;
	int cur = 0;
	c.cpStart[0] = 0; c.cpCount[0] = 1; c.cpNext[0] = 0;
	c.cpRest[0] = cb[0].restitution; c.cpSF[0] = cb[0].staticFriction; c.cpDF[0] = cb[0].dynamicFriction;
	pc = 1;
	V3 mn = cb[0].p, mx = cb[0].p;
	int patchIndex = 0, count = 1;
	for(int i = 1; i < n; i++)
	{
		const Contact& cc = cb[i];
		const Contact& p0 = cb[patchIndex];
		if(cc.staticFriction == p0.staticFriction && cc.dynamicFriction == p0.dynamicFriction && cc.restitution == p0.restitution &&
		   dotS(cc.n, p0.n) >= tol)
		{
			mn = vmin(mn, cc.p);
			mx = vmax(mx, cc.p);
			count++;
		}
		else
		{
			patchIndex = i;
			c.cpCount[cur] = count;
			count = 1;
			c.cpMin[cur] = mn; c.cpMax[cur] = mx;
			cur = pc;
			c.cpStart[pc] = i; c.cpCount[pc] = 1; c.cpNext[pc] = 0;
			c.cpRest[pc] = cc.restitution; c.cpSF[pc] = cc.staticFriction; c.cpDF[pc] = cc.dynamicFriction;
			pc++;
			mn = cc.p; mx = cc.p;
		}
	}
	if(count != 1) c.cpCount[cur] = count;
	c.cpMin[cur] = mn; c.cpMax[cur] = mx;
	c.contactPatchCount = pc;
}

__device__ __forceinline__ void correlatePatches(Correlation& c, const Contact* cb, const Tr& f0, const Tr& f1, float tol)
{
	int fpc = c.frictionPatchCount;
	for(int i = 0; i < c.contactPatchCount; i++)
	{
		const V3 n = cb[c.cpStart[i]].n;
		int j = 0;
		for(; j < fpc && ((dotS(n, c.fpWorldNormal[j]) < tol) || c.fpRest[j] != c.cpRest[i] || c.fpSF[j] != c.cpSF[i] || c.fpDF[j] != c.cpDF[i]); j++)
			;
		if(j == fpc)
		{
			c.fpAnchorCount[fpc] = 0;
			c.fpBroken[fpc] = 0;
			c.fpN0[fpc] = qRotateInvS(f0.q, n);
			c.fpN1[fpc] = qRotateInvS(f1.q, n);
			c.fpQ[fpc] = qMulS(qConj(f0.q), f1.q);
			c.fpSF[fpc] = c.cpSF[i]; c.fpDF[fpc] = c.cpDF[i]; c.fpRest[fpc] = c.cpRest[i];
			c.fpWorldNormal[j] = n;
			c.fpContactCount[fpc] = c.cpCount[i];
			c.fpMin[fpc] = c.cpMin[i]; c.fpMax[fpc] = c.cpMax[i];
			fpc++;
			c.cpNext[i] = -1;
		}
		else
		{
			c.fpMin[j] = vmin(c.fpMin[j], c.cpMin[i]);
			c.fpMax[j] = vmax(c.fpMax[j], c.cpMax[i]);
			c.fpContactCount[j] += c.cpCount[i];
			c.cpNext[i] = c.listHead[j];
		}
		c.listHead[j] = i;
	}
	c.frictionPatchCount = fpc;
}

__device__ __forceinline__ V3 trTransformS(const Tr& t, V3 v) { return add(qRotateS(t.q, v), t.p); }
__device__ __forceinline__ V3 trTransformInvS(const Tr& t, V3 v) { return qRotateInvS(t.q, sub(v, t.p)); }

__device__ __forceinline__ void growPatches(Correlation& c, const Contact* cb, const Tr& f0, const Tr& f1, float thr)
{
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		// a kept patch with two well-spread anchors, or one without contacts,
		// stays as it is (DyFrictionCorrelation.cpp:198-210)
		if(c.fpAnchorCount[i] == 2 || c.listHead[i] == -1)
		{
			const float diag = lenSqS(sub(c.fpMax[i], c.fpMin[i]));
			const float an = lenSqS(sub(c.fpAnchor0[i][0], c.fpAnchor0[i][1]));
			if(c.fpContactCount[i] == 0 || (an * 4.0f) >= diag) continue;
			c.fpAnchorCount[i] = 0;
		}
		V3 wa[2];
		int ac = 0;
		float pointDistSq = 0.0f, d0, d1;
		const float eps = 1e-8f;
		if(c.fpAnchorCount[i] == 1) wa[ac++] = trTransformS(f0, c.fpAnchor0[i][0]);   // a kept anchor stays
		for(int patch = c.listHead[i]; patch != -1; patch = c.cpNext[patch])
		{
			for(int j = 0; j < c.cpCount[patch]; j++)
			{
				const V3 wp = cb[c.cpStart[patch] + j].p;
				if(cb[c.cpStart[patch] + j].sep < thr)
				{
					if(ac == 0) { wa[0] = wp; ac++; }
					else if(ac == 1)
					{
						pointDistSq = lenSqS(sub(wp, wa[0]));
						if(pointDistSq > eps) { wa[1] = wp; ac++; }
					}
					else
					{
						d0 = lenSqS(sub(wp, wa[0]));
						d1 = lenSqS(sub(wp, wa[1]));
						if(d0 > d1)
						{
							if(d0 > pointDistSq) { wa[1] = wp; pointDistSq = d0; }
						}
						else if(d1 > pointDistSq) { wa[0] = wp; pointDistSq = d1; }
					}
				}
			}
		}
		for(int j = c.fpAnchorCount[i]; j < ac; j++)
		{
			c.fpAnchor0[i][j] = trTransformInvS(f0, wa[j]);
			c.fpAnchor1[i][j] = trTransformInvS(f1, wa[j]);
		}
		if(ac == 0) c.fpAnchor0[i][0] = c.fpAnchor1[i][0] = zero3();
		c.fpAnchorCount[i] = ac;
	}
}

// ------------------------------------------------------------- rows
struct PrepParams
{
	float invStepDt, invTotalDt, totalDt, stepDt, bounceThreshold, frictionOffsetThreshold, biasCoefficient, correlationDistance;
};

__device__ __forceinline__ float constructPoint(const M33& s0, const M33& s1, float imn0, float imn1, V3 p0, V3 p1, V3 n, float nv0, float nv1,
                                                V3 av0, V3 av1, float invDtp8, float invStepDt, float totalDt, float invTotalDt,
                                                float restitution, float bounce, const Contact& ct, bool kin0, bool kin1, PointRow& row)
{
	const float zero = 0.0f;
	const float cTarget = dotA(n, zero3());
	const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
	const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
	const float angV0 = dotA(raXn, av0), angV1 = dotA(rbXn, av1);
	const float vrel1 = nv0 + angV0, vrel2 = nv1 + angV1;
	const float vrel = vrel1 - vrel2;
	const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
	const float i0 = dotA(ri0, ri0) * 1.0f, i1 = dotA(ri1, ri1) * 1.0f;
	const float resp0 = imn0 + i0, resp1 = i1 - imn1;
	const float unitResponse = resp0 + resp1;
	const float penetration = ct.sep - 0.0f;
	const bool isSeparated = penetration > zero;
	const float penInvDt = penetration * invTotalDt;
	const bool isGreater2 = (restitution > zero && bounce > vrel) && (-vrel > penInvDt);
	const float ratio = totalDt + (isGreater2 ? penetration / vrel : -totalDt);
	const float recipResponse = unitResponse > zero ? 1.0f / unitResponse : zero;
	const float biasCoeff = -(isSeparated ? invStepDt : invDtp8);
	float totalError = penetration;
	float targetVelocity = cTarget + (isGreater2 ? (-vrel) * restitution : zero);
	totalError = targetVelocity * ratio + totalError;
	if(kin0) targetVelocity = targetVelocity - vrel1;
	if(kin1) targetVelocity = targetVelocity + vrel2;
	row.raXnI = ri0;
	row.rbXnI = ri1;
	row.velMultiplier = recipResponse;
	row.separation = totalError;
	row.biasCoefficient = biasCoeff;
	row.targetVelocity = targetVelocity;
	row.recipResponse = recipResponse;
	row.maxImpulse = FLT_MAX;
	return penetration;
}

// Builds one constraint's rows (createFinalizeSolverContactsStep).  prev: the
// friction patches the pair left last frame (null: fresh friction data);
// written (may be null): the patches it leaves this frame, in patch order.
__device__ __forceinline__ void prepConstraint(const Contact* contacts, int nbContacts, int a, int b, const BodyVel& va, const BodyVel& vb,
                                               const BodyTx& ta, const BodyTx& tb, const BodyData& d0, const BodyData& d1, const Tr& f0,
                                               const Tr& f1, const PrepParams& pp, ConstraintRecord& rec, const FrictionState* prev = nullptr,
                                               FrictionState* written = nullptr)
{
	rec.bodyA = a;
	rec.bodyB = b;
	rec.nbPatches = 0;
	rec.counts = 0;
	if(written) written->count = 0;
	if(nbContacts == 0) return;
	Correlation c;
	getFrictionPatches(c, prev, f0, f1, pp.correlationDistance);
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, pp.frictionOffsetThreshold + 0.0f);

	// row counts first: the rows are packed in this order
	int usedPatches = 0, totalPoints = 0, totalFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		usedPatches++;
		for(int patch = c.listHead[i]; patch != -1; patch = c.cpNext[patch]) totalPoints += c.cpCount[patch];
		totalFriction += c.fpAnchorCount[i] * 2;
	}
	rec.nbPatches = usedPatches;
	rec.counts = totalPoints | (totalFriction << 16);
	PatchRows* patchRows = rec.patch();
	PointRow* pointRows = rec.point();
	FrictionRow* frictionRows = rec.friction();
	float* force = rec.force();
	float* frictionForce = rec.frictionForce();
	int patchOut = 0;
	const bool kin0 = va.kinematic != 0, kin1 = vb.kinematic != 0;
	const float invMass0 = 1.0f * d0.invMass;
	const float invMass1 = (-1.0f) * d1.invMass;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.origLin, lv1 = d1.origLin, av0 = d0.origAng, av1 = d1.origAng;
	const M33& s0 = ta.sqrtInvInertia;
	const M33& s1 = tb.sqrtInvInertia;
	const float invDt = pp.invStepDt;
	const float p8 = fmin_(0.8f, pp.biasCoefficient);
	const float invDtp8 = invDt * p8;
	const float frictionBiasScale = invDt * p8;
	int nPoints = 0, nFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		const int first = c.listHead[i];
		const Contact& base0 = contacts[c.cpStart[first]];
		PatchRows& pr = patchRows[patchOut];
		pr.invMass0 = invMass0;
		pr.invMass1 = -invMass1;
		const V3 n = contacts[c.cpStart[c.listHead[i]]].n;
		const float nLenSq = dotA(n, n);
		const float nv0 = dotA(lv0, n), nv1 = dotA(lv1, n);
		const float imn0 = invMass0 * nLenSq, imn1 = invMass1 * nLenSq;
		pr.normal = n;
		pr.maxPenBias = base0.restitution < 0.0f ? -FLT_MAX : maxPenBias;
		pr.pointStart = nPoints;
		for(int patch = c.listHead[i]; patch != -1; patch = c.cpNext[patch])
			for(int j = 0; j < c.cpCount[patch]; j++)
			{
				constructPoint(s0, s1, imn0, imn1, p0, p1, n, nv0, nv1, av0, av1, invDtp8, invDt, pp.totalDt, pp.invTotalDt, base0.restitution,
				               pp.bounceThreshold, contacts[c.cpStart[patch] + j], kin0, kin1, pointRows[nPoints]);
				force[nPoints] = 0.0f;
				nPoints++;
			}
		pr.nbPoints = nPoints - pr.pointStart;
		pr.staticFriction = base0.staticFriction;
		pr.dynamicFriction = base0.dynamicFriction;
		const int anchors = c.fpAnchorCount[i];
		pr.frictionStart = nFriction;
		pr.nbFriction = anchors ? anchors * 2 : 0;
		if(anchors)
		{
			const V3 linVrel = sub(lv0, lv1);
			const V3 t0f1 = v3(0.0f, -n.z, n.y), t0f2 = v3(-n.y, n.x, 0.0f);
			const V3 t0Fallback = 0.70710678f > fabsf(n.x) ? t0f1 : t0f2;
			V3 t0 = sub(linVrel, scale(n, dotA(n, linVrel)));
			t0 = dotA(t0, t0) > 0.0001f ? t0 : t0Fallback;
			t0 = normalizeA(t0);
			const V3 t1 = normalizeA(cross(n, t0));
			const float nv00 = dotA(lv0, t0), nv01 = dotA(lv1, t0), nv10 = dotA(lv0, t1), nv11 = dotA(lv1, t1);
			const V3 relTr = sub(p0, p1);
			const float frictionScale = anchors == 2 ? 0.5f : 1.0f;
			for(int j = 0; j < anchors; j++)
			{
				const V3 ra = qRotate(f0.q, c.fpAnchor0[i][j]);
				const V3 rb = qRotate(f1.q, c.fpAnchor1[i][j]);
				const V3 error = add(sub(ra, rb), relTr);
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					FrictionRow& fr = frictionRows[nFriction];
					const V3 raXn = cross(ra, t), rbXn = cross(rb, t);
					const V3 ri0 = m33MulV(s0, raXn), ri1 = m33MulV(s1, rbXn);
					const float resp0 = imn0 + dotA(ri0, ri0) * 1.0f;
					const float resp1 = dotA(ri1, ri1) * 1.0f - imn1;
					const float unitResponse = resp0 + resp1;
					const float velMultiplier = unitResponse > 0.0f ? p8 / unitResponse : 0.0f;
					float targetVel = dotA(zero3(), t);
					if(kin0) targetVel = targetVel - ((dir == 0 ? nv00 : nv10) + dotA(raXn, av0));
					if(kin1) targetVel = targetVel + ((dir == 0 ? nv01 : nv11) + dotA(rbXn, av1));
					fr.normal = t;
					fr.error = dotA(error, t);
					fr.raXnI = ri0;
					fr.targetVel = targetVel;
					fr.rbXnI = ri1;
					fr.velMultiplier = velMultiplier;
					fr.frictionScale = frictionScale;
					fr.biasScale = frictionBiasScale;
					frictionForce[nFriction] = 0.0f;
					nFriction++;
				}
			}
		}
		if(written) c.exportPatch(i, written->patches[patchOut]);
		patchOut++;
		if(written) written->count = uint32_t(patchOut);
	}
}

// ------------------------------------------------------------- 4-wide block path, one lane
// PxCreateContactConstraintsTGS builds a header of stride 4 (at most 64
// contacts) with createFinalizeSolverContacts4Step
// (lowleveldynamics/src/DyTGSContactPrepBlock.cpp:1398, rows from
// setupFinalizeSolverConstraints4Step :219) and PxSolveConstraintsTGS solves it
// with solveContact4_Block (:2280).  Its four SIMD lanes never exchange values
// (a lane with fewer patches, points or anchors gets rows of zero response), so
// one lane is the per-constraint computation below, in the block path's own
// evaluation order.  A GB300 thread runs one lane.

// x*x' + y*y' then + z*z' (the block path's V4MulAdd(z, .., V4MulAdd(y, .., V4Mul(x, ..))))
__device__ __forceinline__ float dotXYZ(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// z*z' + y*y' then + x*x'
__device__ __forceinline__ float dotZYX(V3 a, V3 b) { return (a.z * b.z + a.y * b.y) + a.x * b.x; }
// sqrtInvInertia product of the block path: lane-transposed columns dotted with v
__device__ __forceinline__ V3 m33TMulXYZ(const M33& m, V3 v) { return v3(dotXYZ(m.c0, v), dotXYZ(m.c1, v), dotXYZ(m.c2, v)); }
// QuatRotate4V (physx/include/foundation/PxVecQuat.h:208), V4Dot3 = (x + y) + z
__device__ __forceinline__ V3 qRotate4V(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 a = scale(v, w2);
	const V3 u = qv(q);
	const V3 temp = scaleAdd(cross(u, v), q.w, a);
	return scale(scaleAdd(u, dotXYZ(u, v), temp), 2.0f);
}

// Rows of one lane.  blockDynamic: some constraint of the header has a dynamic
// body B (the header-wide isDynamic; passing "this lane's body B is dynamic"
// gives the same values when no body B is kinematic).  keepB: body B's data
// index is 0, so the block solve does not store body B.
__device__ __forceinline__ void prepConstraintBlock(const Contact* contacts, int nbContacts, int a, int b, const BodyVel& va, const BodyVel& vb,
                                                    const BodyTx& ta, const BodyTx& tb, const BodyData& d0, const BodyData& d1, const Tr& f0,
                                                    const Tr& f1, const PrepParams& pp, bool blockDynamic, bool keepB, ConstraintRecord& rec,
                                                    const FrictionState* prev = nullptr, FrictionState* written = nullptr)
{
	rec.bodyA = a;
	rec.bodyB = b;
	rec.nbPatches = 0;
	rec.counts = REC_BLOCK | (keepB ? REC_KEEP_B : 0);
	if(written) written->count = 0;
	if(nbContacts == 0) return;
	Correlation c;
	getFrictionPatches(c, prev, f0, f1, pp.correlationDistance);
	createContactPatches(c, contacts, nbContacts, 0.999f);
	correlatePatches(c, contacts, f0, f1, 0.999f);
	growPatches(c, contacts, f0, f1, pp.frictionOffsetThreshold + 0.0f);
	// The block path then drops the patches that received no contact
	// (createFinalizeSolverContacts4Step, DyTGSContactPrepBlock.cpp:1452-1466)
	// by moving the later list heads and contact counts down -- not the
	// patches themselves, so a later patch's contacts pair with an earlier
	// patch's anchors, and the earlier patches are the ones written out.
	for(int p = c.frictionPatchCount; p > 0; --p)
		if(c.listHead[p - 1] == -1)
		{
			for(int p2 = p; p2 < c.frictionPatchCount; ++p2)
			{
				c.listHead[p2 - 1] = c.listHead[p2];
				c.fpContactCount[p2 - 1] = c.fpContactCount[p2];
			}
			c.frictionPatchCount--;
		}

	int usedPatches = 0, totalPoints = 0, totalFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		usedPatches++;
		for(int patch = c.listHead[i]; patch != -1; patch = c.cpNext[patch]) totalPoints += c.cpCount[patch];
		totalFriction += c.fpAnchorCount[i] * 2;
	}
	rec.nbPatches = usedPatches;
	rec.counts |= totalPoints | (totalFriction << 16);
	PatchRows* patchRows = rec.patch();
	PointRow* pointRows = rec.point();
	FrictionRow* frictionRows = rec.friction();
	float* force = rec.force();
	float* frictionForce = rec.frictionForce();
	// kinematicScale: 1 for a solver body flagged kinematic (statics are); no
	// descriptor of this path has the eKINEMATIC_BODY state
	const float kin0 = va.kinematic ? 1.0f : 0.0f, kin1 = vb.kinematic ? 1.0f : 0.0f;
	const float invMass0D0 = 1.0f * d0.invMass, invMass1D1 = 1.0f * d1.invMass;
	const float angDom0 = 1.0f, angDom1 = 1.0f;
	const float maxPenBias = fmax_(d0.penBiasClamp, d1.penBiasClamp);
	const V3 p0 = f0.p, p1 = f1.p;
	const V3 lv0 = d0.origLin, lv1 = d1.origLin, av0 = d0.origAng, av1 = d1.origAng;
	const M33& s0 = ta.sqrtInvInertia;
	const M33& s1 = tb.sqrtInvInertia;
	const float invDt = pp.invStepDt;
	const float p8 = fmin_(0.8f, pp.biasCoefficient);
	const float frictionBiasScale = invDt * p8;
	const float invDtp8 = invDt * p8;
	const V3 vrel = sub(lv0, lv1);
	int patchOut = 0, nPoints = 0, nFriction = 0;
	for(int i = 0; i < c.frictionPatchCount; i++)
	{
		if(c.fpContactCount[i] == 0) continue;
		const Contact& base0 = contacts[c.cpStart[c.listHead[i]]];
		const float restitution = -base0.restitution;   // negated by the block setup
		PatchRows& pr = patchRows[patchOut];
		pr.invMass0 = invMass0D0;
		pr.invMass1 = invMass1D1;
		const V3 n = base0.n;
		pr.normal = n;
		pr.maxPenBias = maxPenBias;
		const float norVel0 = dotXYZ(n, lv0), norVel1 = dotXYZ(n, lv1);
		const float relNorVel = norVel0 - norVel1;
		pr.pointStart = nPoints;
		for(int patch = c.listHead[i]; patch != -1; patch = c.cpNext[patch])
			for(int j = 0; j < c.cpCount[patch]; j++)
			{
				const Contact& ct = contacts[c.cpStart[patch] + j];
				PointRow& row = pointRows[nPoints];
				const float cTargetNorVel = dotZYX(zero3(), n);
				const V3 ra = sub(ct.p, p0), rb = sub(ct.p, p1);
				const V3 raXn = cross(ra, n), rbXn = cross(rb, n);
				const float relAngVel0 = dotXYZ(raXn, av0), relAngVel1 = dotXYZ(rbXn, av1);
				const V3 dav0 = m33TMulXYZ(s0, raXn);
				float unitResponse = dotZYX(dav0, dav0) * angDom0 + invMass0D0;
				const float vrel0 = norVel0 + relAngVel0, vrel1 = norVel1 + relAngVel1;
				V3 dav1 = zero3();
				if(blockDynamic)
				{
					dav1 = m33TMulXYZ(s1, rbXn);
					unitResponse = unitResponse + (dotZYX(dav1, dav1) * angDom1 + invMass1D1);
				}
				const float vrelD = vrel0 - vrel1;
				float penetration = ct.sep - 0.0f;
				const float penInvDt = penetration * pp.invTotalDt;
				const bool isSeparated = penetration > 0.0f;
				const bool isGreater2 = (0.0f > restitution && pp.bounceThreshold > vrelD) && (-vrelD > penInvDt);
				const float ratio = isGreater2 ? pp.totalDt + penetration / vrelD : 0.0f;
				const float recipResponse = unitResponse > 0.0f ? 1.0f / unitResponse : 0.0f;
				const float targetVelocity = (vrel1 * kin1 + (isGreater2 ? vrelD * restitution : 0.0f)) - vrel0 * kin0;
				penetration = targetVelocity * ratio + penetration;
				row.raXnI = dav0;
				row.rbXnI = dav1;
				row.velMultiplier = recipResponse;
				row.targetVelocity = cTargetNorVel + targetVelocity;
				row.separation = penetration;
				row.biasCoefficient = -(isSeparated ? invDt : invDtp8);
				row.recipResponse = recipResponse;
				row.maxImpulse = FLT_MAX;
				force[nPoints] = 0.0f;
				nPoints++;
			}
		pr.nbPoints = nPoints - pr.pointStart;
		const int anchors = c.fpAnchorCount[i];
		const float coeff = anchors == 2 ? 0.5f : 1.0f;
		pr.staticFriction = base0.staticFriction * coeff;
		pr.dynamicFriction = base0.dynamicFriction * coeff;
		pr.frictionStart = nFriction;
		pr.nbFriction = anchors * 2;
		if(anchors)
		{
			const bool cond = 0.70710678f > fabsf(n.x);
			const V3 fallback = cond ? v3(0.0f, -n.z, n.y) : v3(-n.y, n.x, 0.0f);
			const V3 vs = v3(vrel.x - n.x * relNorVel, vrel.y - n.y * relNorVel, vrel.z - n.z * relNorVel);
			V3 t0 = dotZYX(vs, vs) > 0.0001f ? vs : fallback;
			const float recipLen = 1.0f / sqrtf(dotXYZ(t0, t0));
			t0 = scale(t0, recipLen);
			const V3 t1 = cross(n, t0);
			for(int j = 0; j < anchors; j++)
			{
				const V3 ra = qRotate4V(f0.q, c.fpAnchor0[i][j]);
				const V3 rb = qRotate4V(f1.q, c.fpAnchor1[i][j]);
				const V3 error = sub(add(ra, p0), add(rb, p1));
				for(int dir = 0; dir < 2; dir++)
				{
					const V3 t = dir == 0 ? t0 : t1;
					FrictionRow& fr = frictionRows[nFriction];
					const V3 raXn = cross(ra, t);
					const V3 dav0 = m33TMulXYZ(s0, raXn);
					float resp = dotXYZ(dav0, dav0) * angDom0 + invMass0D0;
					const float vrel0 = ((dotXYZ(t, lv0) + raXn.x * av0.x) + raXn.y * av0.y) + raXn.z * av0.z;
					V3 dav1 = zero3();
					float vrel1 = 0.0f;
					if(blockDynamic)
					{
						const V3 rbXn = cross(rb, t);
						dav1 = m33TMulXYZ(s1, rbXn);
						resp = resp + (dotXYZ(dav1, dav1) * angDom1 + invMass1D1);
						vrel1 = ((dotXYZ(t, lv1) + rbXn.x * av1.x) + rbXn.y * av1.y) + rbXn.z * av1.z;
					}
					fr.normal = t;
					fr.raXnI = dav0;
					fr.rbXnI = dav1;
					fr.velMultiplier = resp > 0.0f ? p8 / resp : 0.0f;
					fr.error = dotXYZ(t, error);
					fr.targetVel = (vrel1 * kin1 + dotXYZ(t, zero3())) - vrel0 * kin0;
					fr.biasScale = frictionBiasScale;
					fr.frictionScale = 1.0f;
					frictionForce[nFriction] = 0.0f;
					nFriction++;
				}
			}
		}
		if(written) c.exportPatch(i, written->patches[patchOut]);
		patchOut++;
		if(written) written->count = uint32_t(patchOut);
	}
}

// ------------------------------------------------------------- solve
// solveContact (DyTGSContactPrep.cpp:1581) for one constraint.  b0/b1 are the
// constraint's two bodies (b1 may be a static/kinematic body, never written
// back when it is not dynamic: its invMass and sqrtInvInertia are zero).
// brokenMask (may be null): bit p set when patch p's friction was clamped in
// this solve (the header's broken flag, written back to the patch's friction
// data after the last iteration).
__device__ __forceinline__ void solveConstraint(ConstraintRecord& rec, BodyVel& b0, BodyVel& b1, bool writeB1, float minPen, float elapsed,
                                                uint32_t* brokenMask = nullptr)
{
	V3 lin0 = b0.lin, lin1 = b1.lin, ang0 = b0.ang, ang1 = b1.ang;
	const V3 angM0 = b0.dAng, angM1 = b1.dAng;
	const V3 relMotion = sub(b0.dLin, b1.dLin);
	const PatchRows* patchRows = rec.patch();
	const PointRow* pointRows = rec.point();
	const FrictionRow* frictionRows = rec.friction();
	float* force = rec.force();
	float* frictionForce = rec.frictionForce();
	for(int p = 0; p < rec.nbPatches; p++)
	{
		const PatchRows pr = patchRows[p];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1;
		const V3 nIM0 = scale(n, invMassA), nIM1 = scale(n, invMassB);
		const float deltaV = dotA(relMotion, n);
		float accumulated = 0.0f;
		for(int i = 0; i < pr.nbPoints; i++)
		{
			const int k = pr.pointStart + i;
			const PointRow c = pointRows[k];
			const float angDelta0 = dotA(angM0, c.raXnI), angDelta1 = dotA(angM1, c.rbXnI);
			const float deltaAng = angDelta0 - angDelta1;
			const float targetVel = c.targetVelocity;
			const float deltaBias = (deltaV + deltaAng) - targetVel * elapsed;
			const float sep = fmax_(minPen, c.separation + deltaBias);
			const float bias = fmin_(-pr.maxPenBias, c.biasCoefficient * sep);
			const V3 v0 = add(mul(lin0, n), mul(ang0, c.raXnI));
			const V3 v1 = add(mul(lin1, n), mul(ang1, c.rbXnI));
			const float normalVel = sumElems(sub(v0, v1));
			const float biasNV = bias * c.recipResponse;
			const float lambda = biasNV - (normalVel - targetVel) * c.velMultiplier;
			const float applied = force[k];
			const float _deltaF = fmax_(lambda, -applied);
			const float _newForce = applied + _deltaF;
			const float newForce = fmin_(_newForce, c.maxImpulse);
			const float deltaF = newForce - applied;
			lin0 = scaleAdd(nIM0, deltaF, lin0);
			lin1 = negScaleSub(nIM1, deltaF, lin1);
			ang0 = scaleAdd(c.raXnI, deltaF * 1.0f, ang0);
			ang1 = negScaleSub(c.rbXnI, deltaF * 1.0f, ang1);
			force[k] = newForce;
			accumulated = accumulated + newForce;
		}
		if(pr.nbFriction)
		{
			const float maxF = pr.staticFriction * accumulated;
			const float maxDynF = pr.dynamicFriction * accumulated;
			const int pairs = pr.nbFriction & 6;
			bool broken = false;
			for(int i = 0; i < pairs; i += 2)
			{
				const int k0 = pr.frictionStart + i, k1 = k0 + 1;
				const FrictionRow& f0 = frictionRows[k0];
				const FrictionRow& f1 = frictionRows[k1];
				const float fs = f0.frictionScale;
				const float biasScale = f0.biasScale;
				float dv0 = (dotA(f0.raXnI, angM0) - dotA(f0.rbXnI, angM1)) + dotA(f0.normal, relMotion);
				float dv1 = (dotA(f1.raXnI, angM0) - dotA(f1.rbXnI, angM1)) + dotA(f1.normal, relMotion);
				dv0 = dv0 - f0.targetVel * elapsed;
				dv1 = dv1 - f1.targetVel * elapsed;
				const float e0 = f0.error + dv0, e1 = f1.error + dv1;
				const float bias0 = e0 * biasScale, bias1 = e1 * biasScale;
				const V3 dl00 = scale(f0.normal, invMassA), dl10 = scale(f0.normal, invMassB);
				const V3 dl01 = scale(f1.normal, invMassA), dl11 = scale(f1.normal, invMassB);
				const float nvel0 = sumElems(sub(add(mul(lin0, f0.normal), mul(ang0, f0.raXnI)), add(mul(lin1, f0.normal), mul(ang1, f0.rbXnI))));
				const float nvel1 = sumElems(sub(add(mul(lin0, f1.normal), mul(ang0, f1.raXnI)), add(mul(lin1, f1.normal), mul(ang1, f1.rbXnI))));
				const float a0 = frictionForce[k0], a1 = frictionForce[k1];
				const float tmp10 = a0 - (bias0 - f0.targetVel) * f0.velMultiplier;
				const float tmp11 = a1 - (bias1 - f1.targetVel) * f1.velMultiplier;
				const float ti0 = tmp10 - nvel0 * f0.velMultiplier;
				const float ti1 = tmp11 - nvel1 * f1.velMultiplier;
				const float total = sqrtf(ti0 * ti0 + ti1 * ti1);
				const bool clamp = total > fs * maxF;
				broken = broken || clamp;
				const float totalClamped = clamp ? fmin_(fs * maxDynF, total) : total;
				const float ratio = total > 0.0f ? totalClamped / total : 0.0f;
				const float nf0 = ti0 * ratio, nf1 = ti1 * ratio;
				const float df0 = nf0 - a0, df1 = nf1 - a1;
				lin0 = scaleAdd(dl00, df0, scaleAdd(dl01, df1, lin0));
				lin1 = negScaleSub(dl10, df0, negScaleSub(dl11, df1, lin1));
				ang0 = scaleAdd(f0.raXnI, df0 * 1.0f, scaleAdd(f1.raXnI, df1 * 1.0f, ang0));
				ang1 = negScaleSub(f0.rbXnI, df0 * 1.0f, negScaleSub(f1.rbXnI, df1 * 1.0f, ang1));
				frictionForce[k0] = nf0;
				frictionForce[k1] = nf1;
			}
			if(brokenMask && broken) *brokenMask |= 1u << p;
		}
	}
	b0.lin = lin0;
	b0.ang = ang0;
	if(writeB1)
	{
		b1.lin = lin1;
		b1.ang = ang1;
	}
}

// One lane of solveContact4_Block (DyTGSContactPrepBlock.cpp:2280): the normal
// velocity's linear part is carried as relVel1 += (invMassA + invMassB) * deltaF
// and the linear velocities move once per patch; friction uses the pre-scaled
// coefficients and a 1e-5 allowance on the static bound, and once an anchor
// pair of a patch exceeds that bound the rest of the patch is clamped to the
// dynamic bound as well.
__device__ __forceinline__ void solveConstraintBlock(ConstraintRecord& rec, BodyVel& b0, BodyVel& b1, bool writeB1, float minPen, float elapsed,
                                                     uint32_t* brokenMask = nullptr)
{
	V3 lin0 = b0.lin, lin1 = b1.lin, ang0 = b0.ang, ang1 = b1.ang;
	const V3 angD0v = b0.dAng, angD1v = b1.dAng;
	const V3 linDelta = sub(b0.dLin, b1.dLin);
	const PatchRows* patchRows = rec.patch();
	const PointRow* pointRows = rec.point();
	const FrictionRow* frictionRows = rec.friction();
	float* force = rec.force();
	float* frictionForce = rec.frictionForce();
	for(int p = 0; p < rec.nbPatches; p++)
	{
		const PatchRows pr = patchRows[p];
		const V3 n = pr.normal;
		const float invMassA = pr.invMass0, invMassB = pr.invMass1;
		const float sumInvMass = invMassA + invMassB;
		float relVel1 = dotXYZ(lin0, n) - dotXYZ(lin1, n);
		const float deltaNormalV = dotXYZ(linDelta, n);
		float accumDeltaF = 0.0f, accumulated = 0.0f;
		for(int i = 0; i < pr.nbPoints; i++)
		{
			const int k = pr.pointStart + i;
			const PointRow c = pointRows[k];
			const float applied = force[k];
			const float normalVel = relVel1 + (dotXYZ(c.raXnI, ang0) - dotXYZ(c.rbXnI, ang1));
			const float deltaAng = dotXYZ(angD0v, c.raXnI) - dotXYZ(angD1v, c.rbXnI);
			const float deltaBias = (deltaNormalV + deltaAng) - c.targetVelocity * elapsed;
			const float sep = fmax_(minPen, c.separation + deltaBias);
			const float bias = fmin_(-pr.maxPenBias, c.biasCoefficient * sep);
			const float _deltaF = fmax_(bias * c.recipResponse - (normalVel - c.targetVelocity) * c.velMultiplier, -applied);
			const float newForce = fmin_(applied + _deltaF, c.maxImpulse);
			const float deltaF = newForce - applied;
			accumDeltaF = accumDeltaF + deltaF;
			relVel1 = sumInvMass * deltaF + relVel1;
			ang0 = add(scale(c.raXnI, deltaF * 1.0f), ang0);
			ang1 = sub(ang1, scale(c.rbXnI, deltaF * 1.0f));
			force[k] = newForce;
			accumulated = accumulated + newForce;
		}
		const float accIM0 = accumDeltaF * invMassA, accIM1 = accumDeltaF * invMassB;
		lin0 = add(scale(n, accIM0), lin0);
		lin1 = sub(lin1, scale(n, accIM1));
		if(pr.nbFriction)
		{
			const float maxF = pr.staticFriction * accumulated + 1e-5f;
			const float maxDynF = pr.dynamicFriction * accumulated;
			bool broken = false;
			for(int i = 0; i < pr.nbFriction; i += 2)
			{
				const int k0 = pr.frictionStart + i, k1 = k0 + 1;
				const FrictionRow& f0 = frictionRows[k0];
				const FrictionRow& f1 = frictionRows[k1];
				const float nv0 = (dotXYZ(lin0, f0.normal) + dotXYZ(f0.raXnI, ang0)) - (dotXYZ(lin1, f0.normal) + dotXYZ(f0.rbXnI, ang1));
				const float nv1 = (dotXYZ(lin0, f1.normal) + dotXYZ(f1.raXnI, ang0)) - (dotXYZ(lin1, f1.normal) + dotXYZ(f1.rbXnI, ang1));
				const float da0 = dotXYZ(angD0v, f0.raXnI) - dotXYZ(angD1v, f0.rbXnI);
				const float da1 = dotXYZ(angD0v, f1.raXnI) - dotXYZ(angD1v, f1.rbXnI);
				const float e0 = f0.error + ((dotXYZ(linDelta, f0.normal) + da0) - f0.targetVel * elapsed);
				const float e1 = f1.error + ((dotXYZ(linDelta, f1.normal) + da1) - f1.targetVel * elapsed);
				const float a0 = frictionForce[k0], a1 = frictionForce[k1];
				const float ti0 = (a0 - (e0 * f0.biasScale - f0.targetVel) * f0.velMultiplier) - nv0 * f0.velMultiplier;
				const float ti1 = (a1 - (e1 * f1.biasScale - f1.targetVel) * f1.velMultiplier) - nv1 * f1.velMultiplier;
				const float total = sqrtf(ti0 * ti0 + ti1 * ti1);
				broken = broken || total > maxF;
				const float totalClamped = broken ? fmin_(total, maxDynF) : total;
				const float ratio = total > 0.0f ? totalClamped / total : 0.0f;
				const float nf0 = ti0 * ratio, nf1 = ti1 * ratio;
				const float df0 = nf0 - a0, df1 = nf1 - a1;
				frictionForce[k0] = nf0;
				frictionForce[k1] = nf1;
				const float im00 = df0 * invMassA, im10 = df0 * invMassB, im01 = df1 * invMassA, im11 = df1 * invMassB;
				lin0 = add(scale(f0.normal, im00), add(scale(f1.normal, im01), lin0));
				lin1 = sub(sub(lin1, scale(f1.normal, im11)), scale(f0.normal, im10));
				ang0 = add(scale(f0.raXnI, df0 * 1.0f), add(scale(f1.raXnI, df1 * 1.0f), ang0));
				ang1 = sub(sub(ang1, scale(f1.rbXnI, df1 * 1.0f)), scale(f0.rbXnI, df0 * 1.0f));
			}
			if(brokenMask && broken) *brokenMask |= 1u << p;
		}
	}
	b0.lin = lin0;
	b0.ang = ang0;
	if(writeB1 && !rec.keepB())
	{
		b1.lin = lin1;
		b1.ang = ang1;
	}
}

// The solve of a constraint record by the path that built it.
__device__ __forceinline__ void solveRecord(ConstraintRecord& rec, BodyVel& b0, BodyVel& b1, bool writeB1, float minPen, float elapsed,
                                            uint32_t* brokenMask = nullptr)
{
	if(rec.isBlock()) solveConstraintBlock(rec, b0, b1, writeB1, minPen, elapsed, brokenMask);
	else solveConstraint(rec, b0, b1, writeB1, minPen, elapsed, brokenMask);
}

// The written friction patch that receives patch p's broken flag.  Per pair
// (single path) it is patch p itself.  A block lane's write-back address
// advances only for the header's patch rows that had friction in any of the
// four lanes (DyTGSContactPrepBlock.cpp:1218-1222): group[0..3] are the
// header's records.
__device__ __forceinline__ int blockBrokenSlot(ConstraintRecord* const* group, int p)
{
	int slot = 0;
	for(int j = 0; j < p; j++)
	{
		bool anyFriction = false;
		for(int l = 0; l < 4; l++)
			if(group[l] && j < group[l]->nbPatches && group[l]->patch()[j].nbFriction > 0) anyFriction = true;
		if(anyFriction) slot++;
	}
	return slot;
}

// integrateCoreStep (DyTGSDynamics.cpp:1403)
__device__ __forceinline__ void integrateStep(BodyVel& v, BodyTx& t, float dt)
{
	const V3 delta = scale(v.lin, dt);
	const V3 unmolested = v.ang;
	const V3 angMotion = m33MulVS(t.sqrtInvInertia, v.ang);
	const float w2 = lenSqS(angMotion);
	t.p = add(t.p, delta);
	if(w2 != 0.0f)
	{
		const float w = sqrtf(w2);
		const float vv = dt * w * 0.5f;
		// sin/cos correctly rounded, which the host C library's sinf/cosf match far
		// more often than the single-precision device functions do
		float s, q;
		sinCosAngle(vv, s, q);
		s /= w;
		const V3 pqr = scale(angMotion, s);
		const Q qv_ = {pqr.x, pqr.y, pqr.z, 0.0f};
		Q r = qMulS(qv_, t.dq);
		r.x += t.dq.x * q; r.y += t.dq.y * q; r.z += t.dq.z * q; r.w += t.dq.w * q;
		const float m = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w);
		const float inv = 1.0f / m;
		t.dq.x = r.x * inv; t.dq.y = r.y * inv; t.dq.z = r.z * inv; t.dq.w = r.w * inv;
	}
	v.dAng = add(v.dAng, scale(unmolested, dt));
	v.dLin = add(v.dLin, delta);
}

// PxIntegrateSolverBodiesTGS (NpImmediateMode.cpp:1719): world angular velocity and new pose
__device__ __forceinline__ void finalizeBody(const BodyVel& v, const BodyTx& t, Tr& pose, V3& angWorld)
{
	angWorld = m33MulVS(t.sqrtInvInertia, v.ang);
	Q q = qMulS(t.dq, pose.q);
	const float m = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
	const float inv = 1.0f / m;
	pose.q.x = q.x * inv; pose.q.y = q.y * inv; pose.q.z = q.z * inv; pose.q.w = q.w * inv;
	pose.p = t.p;
}
} // namespace tgs
} // namespace gbpx
