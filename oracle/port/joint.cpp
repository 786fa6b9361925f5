// ORACLE (test infrastructure, never shipped): CPU restatement of the TGS
// immediate-mode joint (1D constraint) path for rigid bodies:
//   PxCreateJointConstraintsTGS (physx/source/immediatemode/src/NpImmediateMode.cpp:1480) ->
//     setupSolverConstraintStep (lowleveldynamics/src/DyTGSContactPrep.cpp:1939) ->
//       preprocessRows / orthogonalize (lowleveldynamics/src/DyConstraintSetup.cpp:492,213)
//       and the row constants of lowleveldynamics/shared/DyCpuGpu1dConstraint.h
//       (computeMinMaxImpulseOrForceAsImpulse :71, computeJointSpeedTGS :372,
//       computeMaxBiasVelocityTGS :330, compute1dConstraintSolverConstantsTGS :423,
//       raiseInternalFlagsTGS :607, computeBounceVelocity :130)
//   PxSolveConstraintsTGS (NpImmediateMode.cpp:1630) -> solve1DStep
//     (DyTGSContactPrep.cpp:2418), conclude1DStep (:2750), writeBack1DStep (:2837)
// A header of stride 4 whose joints all have rows takes the reference's 4-wide
// path (setupSolverConstraintStep4, DyTGSContactPrepBlock.cpp:1719;
// solve1DStep4 :2957, writeBack1D4 :3418), restated here one lane at a time
// in that path's operation order (solveJointBlock).  The joint rows are the caller's
// (Px1DConstraint); PxConstraintFlag::eIMPROVED_SLERP drive diagonalisation
// is not restated (the caller's flags must not ask for it).
#include "pxmath.h"
#include "tgs_bodies.h"
#include <string.h>
#include <algorithm>
#include <vector>

#define OX extern "C" __attribute__((visibility("default")))

using namespace orc;

namespace
{
// Px1DConstraint (physx/include/PxConstraintDesc.h:194), 80 bytes
struct Row1D
{
	float linear0[3]; float geometricError;
	float angular0[3]; float velocityTarget;
	float linear1[3]; float minImpulse;
	float angular1[3]; float maxImpulse;
	float mod0, mod1;   // spring stiffness, damping / restitution, velocity threshold
	uint16_t flags, solveHint;
	uint32_t pad;
};
static_assert(sizeof(Row1D) == 80, "Px1DConstraint layout");

// Px1DConstraintFlag, PxConstraintSolveHint
enum { F_SPRING = 1, F_ACCEL_SPRING = 2, F_RESTITUTION = 4, F_KEEPBIAS = 8, F_OUTPUT_FORCE = 16, F_HAS_DRIVE_LIMIT = 32, F_ANGULAR = 64 };
enum { H_EQUALITY = 2048, H_INEQUALITY = 2049, H_ROT_EQUALITY = 1024, H_ROT_INEQUALITY = 1025 };
// solver row flags (lowleveldynamics/src/DySolverConstraintTypes.h:60)
enum { S_OUTPUT_FORCE = 2, S_KEEP_BIAS = 4, S_ROT_EQ = 8, S_ORTHO_TARGET = 16, S_SPRING = 32, S_INEQUALITY = 64, S_ACCEL_SPRING = 128 };
enum { TYPE_RB_1D = 2, TYPE_BLOCK_1D = 8 };
const int MAX_ROWS = 12;

// SolverConstraint1DStep fields
struct SolverRow
{
	V3 lin0, lin1, ang0, ang1;
	float error, biasScale, velMultiplier, velTarget, minImpulse, maxImpulse, appliedForce, maxBias, recipResponse;
	uint32_t flags;
	float angularErrorScale;   // getUseAngularError(): 1 or 0
};
// SolverConstraint1DHeaderStep fields
struct JointRows
{
	int bodyA, bodyB;
	bool block;                // a lane of a 4-wide header (the block path's arithmetic)
	int count;
	float invMass0, invMass1, angScale0, angScale1;   // angScale1: -angular1 (per-pair header), +angular1 (4-wide)
	float linBreakImpulse, angBreakImpulse;
	bool breakable;
	V3 body0WorldOffset, rA, rB;
	V3 orthoAxis0[3], orthoAxis1[3];
	float orthoRecipResponse[3], orthoError[3];
	std::vector<SolverRow> rows;
};

struct V4f { float x, y, z, w; };
// the 4-wide path's sums: V4MulAdd chains give x + (y + z) (V4Dot3,
// DyTGSContactPrepBlock.cpp:2952) and QuatRotate4's dot gives (x + y) + z
static inline float dotX_YZ(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
static inline float dotXY_Z(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 m33TMulXY_Z(const M33& m, V3 v) { return v3(dotXY_Z(m.c0, v), dotXY_Z(m.c1, v), dotXY_Z(m.c2, v)); }
// QuatRotate4 (DyTGSContactPrepBlock.cpp:57): 2 (v (w^2 - 1/2) + (u x v) w + u (u.v))
static inline V3 qRotate4(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 u = v3(q.x, q.y, q.z);
	const V3 temp = add(scale(cross(u, v), q.w), scale(v, w2));
	return scale(add(scale(u, dotXY_Z(u, v)), temp), 2.0f);
}
static inline V4f v4(float x, float y, float z, float w) { V4f r = {x, y, z, w}; return r; }

// ---------------------------------------------------------------- preprocessRows
struct MassProps { float invMass0, invMass1, invInertiaScale0, invInertiaScale1; };

// orthogonalize (DyConstraintSetup.cpp:213): Gram-Schmidt of the rows over the
// mass metric, the geometric error riding in linear0's W lane and the velocity
// target in angular0's; equality rows become base vectors for all later rows.
void orthogonalize(Row1D** row, V4f* angSqrt0, V4f* angSqrt1, int rowCount, int eqRowCount, const MassProps& m)
{
	V4f lin0m[6], ang0m[6], lin0AndG[6], ang0AndT[6];
	V3 lin1m[6], ang1m[6], lin1[6], ang1[6];
	for(int i = 0; i < rowCount; i++)
	{
		Row1D& r = *row[i];
		V4f l0AndG = v4(r.linear0[0], r.linear0[1], r.linear0[2], r.geometricError);
		V4f a0AndT = v4(r.angular0[0], r.angular0[1], r.angular0[2], r.velocityTarget);
		V3 l1 = v3(r.linear1[0], r.linear1[1], r.linear1[2]);
		V3 a1 = v3(r.angular1[0], r.angular1[1], r.angular1[2]);
		V4f aL0 = angSqrt0[i], aL1 = angSqrt1[i];
		const int elim = std::min(i, eqRowCount);
		for(int j = 0; j < elim; j++)
		{
			const V3 s0 = v3(l1.x * lin1m[j].x + l0AndG.x * lin0m[j].x, l1.y * lin1m[j].y + l0AndG.y * lin0m[j].y,
			                 l1.z * lin1m[j].z + l0AndG.z * lin0m[j].z);
			const V3 s1 = v3(aL1.x * ang1m[j].x + aL0.x * ang0m[j].x, aL1.y * ang1m[j].y + aL0.y * ang0m[j].y,
			                 aL1.z * ang1m[j].z + aL0.z * ang0m[j].z);
			const float t = sumElems(add(s0, s1));
			l0AndG = v4(l0AndG.x - lin0AndG[j].x * t, l0AndG.y - lin0AndG[j].y * t, l0AndG.z - lin0AndG[j].z * t, l0AndG.w - lin0AndG[j].w * t);
			a0AndT = v4(a0AndT.x - ang0AndT[j].x * t, a0AndT.y - ang0AndT[j].y * t, a0AndT.z - ang0AndT[j].z * t, a0AndT.w - ang0AndT[j].w * t);
			l1 = sub(l1, scale(lin1[j], t));
			a1 = sub(a1, scale(ang1[j], t));
			aL0 = v4(aL0.x - angSqrt0[j].x * t, aL0.y - angSqrt0[j].y * t, aL0.z - angSqrt0[j].z * t, aL0.w - angSqrt0[j].w * t);
			aL1 = v4(aL1.x - angSqrt1[j].x * t, aL1.y - angSqrt1[j].y * t, aL1.z - angSqrt1[j].z * t, aL1.w - angSqrt1[j].w * t);
		}
		r.linear0[0] = l0AndG.x; r.linear0[1] = l0AndG.y; r.linear0[2] = l0AndG.z; r.geometricError = l0AndG.w;
		r.angular0[0] = a0AndT.x; r.angular0[1] = a0AndT.y; r.angular0[2] = a0AndT.z; r.velocityTarget = a0AndT.w;
		r.linear1[0] = l1.x; r.linear1[1] = l1.y; r.linear1[2] = l1.z;
		r.angular1[0] = a1.x; r.angular1[1] = a1.y; r.angular1[2] = a1.z;
		angSqrt0[i] = aL0;
		angSqrt1[i] = aL1;
		if(i < eqRowCount)
		{
			lin0AndG[i] = l0AndG;
			ang0AndT[i] = a0AndT;
			lin1[i] = l1;
			ang1[i] = a1;
			const V3 l0 = v3(l0AndG.x, l0AndG.y, l0AndG.z);
			const V3 l0m = scale(l0, m.invMass0);
			const V3 l1m = scale(l1, m.invMass1);
			const V4f a0m = v4(aL0.x * m.invInertiaScale0, aL0.y * m.invInertiaScale0, aL0.z * m.invInertiaScale0, aL0.w * m.invInertiaScale0);
			const V4f a1m = v4(aL1.x * m.invInertiaScale1, aL1.y * m.invInertiaScale1, aL1.z * m.invInertiaScale1, aL1.w * m.invInertiaScale1);
			const V3 s0 = v3(l0.x * l0m.x + l1.x * l1m.x, l0.y * l0m.y + l1.y * l1m.y, l0.z * l0m.z + l1.z * l1m.z);
			const V3 s1 = v3(a0m.x * aL0.x + a1m.x * aL1.x, a0m.y * aL0.y + a1m.y * aL1.y, a0m.z * aL0.z + a1m.z * aL1.z);
			const float s = sumElems(add(s0, s1));
			const float a = s > 0.0f ? 1.0f / s : 0.0f;
			lin0m[i] = v4(l0m.x * a, l0m.y * a, l0m.z * a, 0.0f);
			ang0m[i] = v4(a0m.x * a, a0m.y * a, a0m.z * a, 0.0f);
			lin1m[i] = scale(l1m, a);
			ang1m[i] = scale(v3(a1m.x, a1m.y, a1m.z), a);
		}
	}
}

// preprocessRows (DyConstraintSetup.cpp:492): stable insertion sort by solve
// hint, I^(-1/2) * angular per row, then orthogonalisation of the equality
// groups (hint >> 8 == 4: rotational, == 8: linear).
void preprocessRows(Row1D** sorted, Row1D* rows, V4f* angSqrt0, V4f* angSqrt1, int rowCount, const M33& sqrtInv0, const M33& sqrtInv1,
                    float invMass0, float invMass1, const float* ims, bool disablePreprocessing)
{
	for(int i = 0; i < rowCount; i++)
	{
		Row1D* r = rows + i;
		int j = i;
		for(; j > 0 && r->solveHint < sorted[j - 1]->solveHint; j--) sorted[j] = sorted[j - 1];
		sorted[j] = r;
	}
	for(int i = 0; i < rowCount; i++)
	{
		const V3 d0 = m33MulV(sqrtInv0, v3(sorted[i]->angular0[0], sorted[i]->angular0[1], sorted[i]->angular0[2]));
		const V3 d1 = m33MulV(sqrtInv1, v3(sorted[i]->angular1[0], sorted[i]->angular1[1], sorted[i]->angular1[2]));
		angSqrt0[i] = v4(d0.x, d0.y, d0.z, 0.0f);
		angSqrt1[i] = v4(d1.x, d1.y, d1.z, 0.0f);
	}
	if(disablePreprocessing) return;
	const MassProps m = {invMass0 * ims[0], invMass1 * ims[2], ims[1], ims[3]};
	for(int i = 0; i < rowCount;)
	{
		const uint32_t group = sorted[i]->solveHint >> 8;
		const int start = i++;
		while(i < rowCount && uint32_t(sorted[i]->solveHint >> 8) == group) i++;
		if(group == 4 || group == 8)
		{
			int bCount = start;
			for(; bCount < i && (sorted[bCount]->solveHint & 255) == 0; bCount++)
				;
			orthogonalize(sorted + start, angSqrt0 + start, angSqrt1 + start, i - start, bCount - start, m);
		}
	}
}

// ---------------------------------------------------------------- row constants
float bounceVelocity(uint32_t flags, float jointSpeed, float threshold, float restitution, float geometricError)
{
	const float bounceVel = jointSpeed * (-restitution);
	if((flags & F_RESTITUTION) && (-jointSpeed > threshold) && ((bounceVel * geometricError) <= 0.0f)) return bounceVel;
	return 0.0f;
}

float maxBiasVelocity(uint32_t flags, float jointSpeed, float threshold, float restitution, float geometricError, float lengthScale, float recipSimDt)
{
	if(flags & F_SPRING) return FLT_MAX;
	if(bounceVelocity(flags, jointSpeed, threshold, restitution, geometricError) != 0.0f) return 0.0f;
	if(flags & F_ANGULAR) return recipSimDt * 0.75f;
	return recipSimDt * 15.0f * lengthScale;
}

// compute1dConstraintSolverConstantsTGS: biasScale, error, velMultiplier, targetVel
void solverConstants(const Row1D& c, float jointSpeed, float initJointSpeed, float unitResponse, float recipUnitResponse, float erp, float stepDt,
                     float recipStepDt, SolverRow& s)
{
	const uint32_t flags = c.flags;
	if(flags & F_SPRING)
	{
		const float stiffness = c.mod0, damping = c.mod1;
		const float a = stepDt * (stepDt * stiffness + damping);
		const float b = stepDt * (damping * c.velocityTarget);
		if(flags & F_ACCEL_SPRING)
		{
			const float x = 1.0f / (1.0f + a);
			const float biasScale = -x * stiffness * stepDt * recipUnitResponse;
			const float velMultiplier = -x * a * recipUnitResponse;
			s.biasScale = biasScale;
			s.error = biasScale * c.geometricError;
			s.velMultiplier = velMultiplier;
			s.velTarget = x * b * recipUnitResponse - velMultiplier * initJointSpeed;
		}
		else
		{
			const float x = 1.0f / (1.0f + a * unitResponse);
			const float biasScale = -x * stiffness * stepDt;
			const float velMultiplier = -x * a;
			s.biasScale = biasScale;
			s.error = biasScale * c.geometricError;
			s.velMultiplier = velMultiplier;
			s.velTarget = x * b - velMultiplier * initJointSpeed;
		}
		return;
	}
	const float bounceVel = bounceVelocity(flags, jointSpeed, c.mod1, c.mod0, c.geometricError);
	const float velMultiplier = -1.0f;
	if(bounceVel != 0.0f)
	{
		s.biasScale = 0.0f;
		s.error = 0.0f;
		s.velMultiplier = velMultiplier;
		s.velTarget = bounceVel - velMultiplier * initJointSpeed;
	}
	else
	{
		const float biasScale = -recipStepDt * erp;
		s.biasScale = biasScale;
		s.error = c.geometricError * biasScale;
		s.velMultiplier = velMultiplier;
		s.velTarget = c.velocityTarget - velMultiplier * initJointSpeed;
	}
}

uint32_t internalFlags(uint32_t flags, uint32_t hint)
{
	uint32_t f = 0;
	if(flags & F_SPRING) f |= S_SPRING;
	if(flags & F_ACCEL_SPRING) f |= S_ACCEL_SPRING;
	if(flags & F_OUTPUT_FORCE) f |= S_OUTPUT_FORCE;
	if(flags & F_KEEPBIAS) f |= S_KEEP_BIAS;
	if(hint & 1) f |= S_INEQUALITY;
	return f;
}

struct JointIn
{
	int a, b;
	const BodyVel* v0; const BodyVel* v1;
	const BodyTx* t0; const BodyTx* t1;
	const BodyData* d0; const BodyData* d1;
	Tr frame0, frame1;
	const float* params;   // 20 floats: ims, cA2w, cB2w, body0WorldOffset, breaks, min response, flags
	Row1D* rows;
	int numRows;
};

// setupSolverConstraintStep (DyTGSContactPrep.cpp:1939), rigid bodies only.
void setupJoint(const JointIn& in, bool block, float stepDt, float simDt, float recipStepDt, float recipSimDt, float lengthScale, float biasCoefficient,
                JointRows& out)
{
	out.block = block;
	const float* ims = in.params;
	const uint32_t pflags = uint32_t(in.params[16]);
	const bool disablePre = (pflags & 1u) != 0, driveLimitsAreForces = (pflags & 4u) != 0;
	out.bodyA = in.a;
	out.bodyB = in.b;
	out.count = in.numRows;
	out.invMass0 = in.d0->invMass * ims[0];
	out.invMass1 = in.d1->invMass * ims[2];
	out.angScale0 = ims[1];
	out.angScale1 = block ? ims[3] : -ims[3];   // the 4-wide header keeps it positive
	out.body0WorldOffset = v3(in.params[10], in.params[11], in.params[12]);
	out.linBreakImpulse = in.params[13] * simDt;
	out.angBreakImpulse = in.params[14] * simDt;
	out.breakable = in.params[13] != FLT_MAX || in.params[14] != FLT_MAX;
	out.rA = sub(v3(in.params[4], in.params[5], in.params[6]), in.frame0.p);
	out.rB = sub(v3(in.params[7], in.params[8], in.params[9]), in.frame1.p);
	for(int k = 0; k < 3; k++)
	{
		out.orthoAxis0[k] = out.orthoAxis1[k] = zero3();
		out.orthoRecipResponse[k] = out.orthoError[k] = 0.0f;
	}
	out.rows.assign(size_t(in.numRows), SolverRow());
	if(in.numRows == 0) return;
	for(int i = 0; i < in.numRows; i++)
	{
		Row1D& r = in.rows[i];
		if(r.flags & F_ANGULAR)
		{
			if(r.solveHint == H_EQUALITY) r.solveHint = H_ROT_EQUALITY;
			else if(r.solveHint == H_INEQUALITY) r.solveHint = H_ROT_INEQUALITY;
		}
	}
	Row1D* sorted[MAX_ROWS];
	V4f angSqrt0[MAX_ROWS], angSqrt1[MAX_ROWS];
	preprocessRows(sorted, in.rows, angSqrt0, angSqrt1, in.numRows, in.t0->sqrtInvInertia, in.t1->sqrtInvInertia, in.d0->invMass, in.d1->invMass,
	               ims, disablePre);
	const float erp = 0.5f * biasCoefficient;
	int orthoCount = 0;
	for(int i = 0; i < in.numRows; i++)
	{
		const Row1D& c = *sorted[i];
		SolverRow& s = out.rows[size_t(i)];
		const float driveScale = ((c.flags & F_HAS_DRIVE_LIMIT) && driveLimitsAreForces) ? simDt : 1.0f;
		s.lin0 = v3(c.linear0[0], c.linear0[1], c.linear0[2]);
		s.lin1 = v3(c.linear1[0], c.linear1[1], c.linear1[2]);
		s.ang0 = v3(c.angular0[0], c.angular0[1], c.angular0[2]);
		s.ang1 = v3(c.angular1[0], c.angular1[1], c.angular1[2]);
		s.minImpulse = c.minImpulse * driveScale;
		s.maxImpulse = c.maxImpulse * driveScale;
		s.flags = 0;
		s.appliedForce = 0.0f;
		s.angularErrorScale = 1.0f;
		const V3 aS0 = v3(angSqrt0[i].x, angSqrt0[i].y, angSqrt0[i].z), aS1 = v3(angSqrt1[i].x, angSqrt1[i].y, angSqrt1[i].z);
		float unitResponse, vel0, vel1;
		if(!block)
		{
			const float linSumMass = lenSqS(s.lin0) * in.d0->invMass * ims[0] + lenSqS(s.lin1) * in.d1->invMass * ims[2];
			const float resp0 = lenSqS(aS0) * ims[1];
			const float resp1 = lenSqS(aS1) * ims[3];
			unitResponse = resp0 + resp1 + linSumMass;
			vel0 = dotS(in.d0->origLin, s.lin0) + dotS(in.d0->origAng, s.ang0);
			vel1 = dotS(in.d1->origLin, s.lin1) + dotS(in.d1->origAng, s.ang1);
		}
		else
		{
			// setupSolverConstraintStep4 (DyTGSContactPrepBlock.cpp:2087-2106): pre-scaled
			// masses, per-body sums, and body B's angular speed taken along I^(-1/2) angular1
			unitResponse = (lenSqS(s.lin0) * out.invMass0 + lenSqS(aS0) * ims[1]) + (lenSqS(s.lin1) * out.invMass1 + lenSqS(aS1) * ims[3]);
			vel0 = dotX_YZ(s.lin0, in.d0->origLin) + dotX_YZ(s.ang0, in.d0->origAng);
			vel1 = dotX_YZ(s.lin1, in.d1->origLin) + dotX_YZ(aS1, in.d1->origAng);
		}
		float initJointSpeed = 0.0f;
		if(in.v0->kinematic) initJointSpeed -= vel0;
		if(in.v1->kinematic) initJointSpeed += vel1;
		const float jointSpeed = vel0 - vel1;
		if(!(c.flags & F_ANGULAR))
		{
			s.ang0 = zero3();
			s.ang1 = zero3();
			s.angularErrorScale = 0.0f;
		}
		const float minResponse = in.params[15];
		const float recipUnitResponse = unitResponse <= minResponse ? 0.0f : 1.0f / unitResponse;
		s.recipResponse = recipUnitResponse;
		s.maxBias = maxBiasVelocity(c.flags, jointSpeed, c.mod1, c.mod0, c.geometricError, lengthScale, recipSimDt);
		solverConstants(c, jointSpeed, initJointSpeed, unitResponse, recipUnitResponse, erp, stepDt, recipStepDt, s);
		s.flags = internalFlags(c.flags, c.solveHint);
		if(!disablePre)
		{
			if(c.solveHint == H_ROT_EQUALITY)
			{
				s.flags |= S_ROT_EQ;
				out.orthoAxis0[orthoCount] = v3(angSqrt0[i].x * ims[1], angSqrt0[i].y * ims[1], angSqrt0[i].z * ims[1]);
				out.orthoRecipResponse[orthoCount] = recipUnitResponse;
				out.orthoAxis1[orthoCount] = v3(angSqrt1[i].x * ims[3], angSqrt1[i].y * ims[3], angSqrt1[i].z * ims[3]);
				out.orthoError[orthoCount] = c.geometricError;
				orthoCount++;
			}
			else if(c.solveHint & H_EQUALITY)
				s.flags |= S_ORTHO_TARGET;
		}
	}
}

// ---------------------------------------------------------------- solve
// solve1DStep (DyTGSContactPrep.cpp:2418)
void solveJoint(JointRows& j, BodyVel* vels, const BodyTx* txs, float elapsed)
{
	if(j.count == 0) return;
	BodyVel& b0 = vels[j.bodyA];
	BodyVel& b1 = vels[j.bodyB];
	const BodyTx& t0 = txs[j.bodyA];
	const BodyTx& t1 = txs[j.bodyB];
	V3 linVel0 = b0.lin, linVel1 = b1.lin, angState0 = b0.ang, angState1 = b1.ang;
	const V3 ra = qRotate(t0.dq, j.rA), rb = qRotate(t1.dq, j.rB);
	const V3 lin0 = b0.dLin, ang0 = b0.dAng, lin1 = b1.dLin, ang1 = b1.dAng;
	const V3 raMotion = sub(add(ra, lin0), j.rA);
	const V3 rbMotion = sub(add(rb, lin1), j.rB);
	float orthoErr[3];
	for(int k = 0; k < 3; k++) orthoErr[k] = j.orthoError[k] + (dotA(j.orthoAxis0[k], ang0) - dotA(j.orthoAxis1[k], ang1));
	for(int i = 0; i < j.count; i++)
	{
		SolverRow& c = j.rows[size_t(i)];
		const V3 cangVel0 = add(c.ang0, cross(ra, c.lin0));
		const V3 cangVel1 = add(c.ang1, cross(rb, c.lin1));
		float error = c.error;
		const float minBias = -((c.flags & S_INEQUALITY) ? FLT_MAX : c.maxBias);
		V3 raXnI = m33MulV(t0.sqrtInvInertia, cangVel0);
		V3 rbXnI = m33MulV(t1.sqrtInvInertia, cangVel1);
		if(c.flags & S_ORTHO_TARGET)
		{
			float proj[3];
			for(int k = 0; k < 3; k++)
				proj[k] = sumElems(add(mul(raXnI, j.orthoAxis0[k]), mul(rbXnI, j.orthoAxis1[k]))) * j.orthoRecipResponse[k];
			const V3 delta0 = add(scale(j.orthoAxis0[0], proj[0]), add(scale(j.orthoAxis0[1], proj[1]), scale(j.orthoAxis0[2], proj[2])));
			const V3 delta1 = add(scale(j.orthoAxis1[0], proj[0]), add(scale(j.orthoAxis1[1], proj[1]), scale(j.orthoAxis1[2], proj[2])));
			raXnI = sub(raXnI, delta0);
			rbXnI = sub(rbXnI, delta1);
			const float orthoBasisError = c.biasScale * (orthoErr[0] * proj[0] + (orthoErr[1] * proj[1] + orthoErr[2] * proj[2]));
			error = error - orthoBasisError;
		}
		const bool spring = (c.flags & S_SPRING) != 0;
		const float deltaAng = c.angularErrorScale * (dotA(raXnI, ang0) - dotA(rbXnI, ang1));
		const float deltaLin = dotA(c.lin0, raMotion) - dotA(c.lin1, rbMotion);
		const float motion = deltaLin + deltaAng;
		const float errorChange = spring ? motion : motion - c.velTarget * elapsed;
		const float resp0 = j.invMass0 * dotA(c.lin0, c.lin0) + sumElems(mul(scale(raXnI, j.angScale0), raXnI));
		const float resp1 = j.invMass1 * dotA(c.lin1, c.lin1) - sumElems(mul(scale(rbXnI, j.angScale1), rbXnI));
		const float response = resp0 + resp1;
		const float recipResponse = response > 0.0f ? 1.0f / response : 0.0f;
		const float vMul = spring ? c.velMultiplier : recipResponse * c.velMultiplier;
		const float bias = fclamp(errorChange * c.biasScale + error, minBias, c.maxBias);
		const float constant = spring ? bias + c.velTarget : recipResponse * (bias + c.velTarget);
		const V3 v0 = add(mul(linVel0, c.lin0), mul(angState0, raXnI));
		const V3 v1 = add(mul(linVel1, c.lin1), mul(angState1, rbXnI));
		const float normalVel = sumElems(sub(v0, v1));
		const float unclamped = c.appliedForce + (vMul * normalVel + constant);
		const float clamped = fclamp(unclamped, c.minImpulse, c.maxImpulse);
		const float deltaF = clamped - c.appliedForce;
		c.appliedForce = clamped;
		linVel0 = add(scale(c.lin0, deltaF * j.invMass0), linVel0);
		linVel1 = sub(linVel1, scale(c.lin1, deltaF * j.invMass1));
		angState0 = add(scale(raXnI, deltaF * j.angScale0), angState0);
		angState1 = add(scale(rbXnI, deltaF * j.angScale1), angState1);
	}
	b0.lin = linVel0; b0.ang = angState0;
	b1.lin = linVel1; b1.ang = angState1;
}

// One lane of solve1DStep4 (DyTGSContactPrepBlock.cpp:2957); the lane's padding
// rows (beyond its own count) apply no impulse and are skipped.
void solveJointBlock(JointRows& j, BodyVel* vels, const BodyTx* txs, float elapsed)
{
	if(j.count == 0) return;
	BodyVel& b0 = vels[j.bodyA];
	BodyVel& b1 = vels[j.bodyB];
	const BodyTx& t0 = txs[j.bodyA];
	const BodyTx& t1 = txs[j.bodyB];
	V3 linVel0 = b0.lin, linVel1 = b1.lin, angState0 = b0.ang, angState1 = b1.ang;
	const V3 ra = qRotate4(t0.dq, j.rA), rb = qRotate4(t1.dq, j.rB);
	const V3 dAng0 = b0.dAng, dAng1 = b1.dAng;
	const V3 raMotion = sub(add(ra, b0.dLin), j.rA);
	const V3 rbMotion = sub(add(rb, b1.dLin), j.rB);
	float orthoErr[3];
	for(int k = 0; k < 3; k++) orthoErr[k] = j.orthoError[k] + (dotX_YZ(j.orthoAxis0[k], dAng0) - dotX_YZ(j.orthoAxis1[k], dAng1));
	const float mass0 = j.invMass0, mass1 = j.invMass1, scale0 = j.angScale0, scale1 = j.angScale1;
	for(int i = 0; i < j.count; i++)
	{
		SolverRow& c = j.rows[size_t(i)];
		const V3 cangVel0 = add(c.ang0, cross(ra, c.lin0));
		const V3 cangVel1 = add(c.ang1, cross(rb, c.lin1));
		const float coef = (c.flags & S_ORTHO_TARGET) ? 1.0f : 0.0f;
		V3 d0 = m33TMulXY_Z(t0.sqrtInvInertia, cangVel0);
		V3 d1 = m33TMulXY_Z(t1.sqrtInvInertia, cangVel1);
		float err = c.error;
		{
			float proj[3];
			for(int k = 0; k < 3; k++)
			{
				const V3 a0 = j.orthoAxis0[k], a1 = j.orthoAxis1[k];
				proj[k] = (a0.x * d0.x + (a0.y * d0.y + (a0.z * d0.z + (a1.x * d1.x + (a1.y * d1.y + a1.z * d1.z))))) * j.orthoRecipResponse[k];
			}
			const V3* A0 = j.orthoAxis0;
			const V3* A1 = j.orthoAxis1;
			const V3 delta0 = v3(A0[0].x * proj[0] + (A0[1].x * proj[1] + A0[2].x * proj[2]), A0[0].y * proj[0] + (A0[1].y * proj[1] + A0[2].y * proj[2]),
			                     A0[0].z * proj[0] + (A0[1].z * proj[1] + A0[2].z * proj[2]));
			const V3 delta1 = v3(A1[0].x * proj[0] + (A1[1].x * proj[1] + A1[2].x * proj[2]), A1[0].y * proj[0] + (A1[1].y * proj[1] + A1[2].y * proj[2]),
			                     A1[0].z * proj[0] + (A1[1].z * proj[1] + A1[2].z * proj[2]));
			d0 = sub(d0, scale(delta0, coef));
			d1 = sub(d1, scale(delta1, coef));
			const float orthoBasisError = c.biasScale * (orthoErr[0] * proj[0] + (orthoErr[1] * proj[1] + orthoErr[2] * proj[2]));
			err = err - orthoBasisError * coef;
		}
		const bool spring = (c.flags & S_SPRING) != 0;
		const float deltaAng = c.angularErrorScale * (dotX_YZ(d0, dAng0) - dotX_YZ(d1, dAng1));
		const float deltaLin = dotX_YZ(c.lin0, raMotion) - dotX_YZ(c.lin1, rbMotion);
		const float motion = deltaLin + deltaAng;
		const float errorChange = spring ? motion : motion - c.velTarget * elapsed;
		const float resp0 = mass0 * dotX_YZ(c.lin0, c.lin0) + scale0 * dotX_YZ(d0, d0);
		const float resp1 = mass1 * dotX_YZ(c.lin1, c.lin1) + scale1 * dotX_YZ(d1, d1);
		const float response = resp0 + resp1;
		const float recipResponse = response > 0.0f ? 1.0f / response : 0.0f;
		const float vMul = spring ? c.velMultiplier : recipResponse * c.velMultiplier;
		const float minBias = -((c.flags & S_INEQUALITY) ? FLT_MAX : c.maxBias);
		const float bias = fclamp(errorChange * c.biasScale + err, minBias, c.maxBias);
		const float constant = spring ? bias + c.velTarget : recipResponse * (bias + c.velTarget);
		const float normalVel = (dotX_YZ(c.lin0, linVel0) - dotX_YZ(c.lin1, linVel1)) + (dotX_YZ(d0, angState0) - dotX_YZ(d1, angState1));
		const float unclamped = c.appliedForce + (vMul * normalVel + constant);
		const float clamped = fclamp(unclamped, c.minImpulse, c.maxImpulse);
		const float deltaF = clamped - c.appliedForce;
		c.appliedForce = clamped;
		const float fm0 = deltaF * mass0, fm1 = deltaF * mass1, fa0 = deltaF * scale0, fa1 = deltaF * scale1;
		linVel0 = add(scale(c.lin0, fm0), linVel0);
		linVel1 = sub(linVel1, scale(c.lin1, fm1));
		angState0 = add(scale(d0, fa0), angState0);
		angState1 = sub(angState1, scale(d1, fa1));
	}
	b0.lin = linVel0; b0.ang = angState0;
	b1.lin = linVel1; b1.ang = angState1;
}

// conclude1DStep (DyTGSContactPrep.cpp:2750)
void concludeJoint(JointRows& j)
{
	for(int i = 0; i < j.count; i++)
	{
		SolverRow& c = j.rows[size_t(i)];
		if(!(c.flags & S_KEEP_BIAS)) { c.biasScale = 0.0f; c.error = 0.0f; }
		if(c.flags & S_SPRING) { c.velMultiplier = 0.0f; c.biasScale = 0.0f; c.error = 0.0f; c.velTarget = 0.0f; }
	}
}

// writeBack1DStep (DyTGSContactPrep.cpp:2837): impulse of the rows that output force
void writeBackJoint(const JointRows& j, float* force, uint32_t* broken)
{
	V3 lin = zero3(), ang = zero3();
	if(j.block)
	{
		// writeBack1D4 (DyTGSContactPrepBlock.cpp:3418): angular part from angular0
		// alone, and its body0WorldOffset term as the 4-wide code forms it
		for(int i = 0; i < j.count; i++)
		{
			const SolverRow& c = j.rows[size_t(i)];
			const float f = (c.flags & S_OUTPUT_FORCE) ? c.appliedForce : 0.0f;
			lin = add(scale(c.lin0, f), lin);
			ang = add(scale(c.ang0, f), ang);
		}
		const V3 o = j.body0WorldOffset;
		ang = v3(ang.x - (o.y * lin.z - o.x * lin.y), ang.y - (o.z * lin.x - o.y * lin.z), ang.z - (o.x * lin.y - o.z * lin.x));
		force[0] = lin.x; force[1] = lin.y; force[2] = lin.z;
		force[3] = ang.x; force[4] = ang.y; force[5] = ang.z;
		*broken = j.breakable ? uint32_t(sqrtf(lenSqS(lin)) > j.linBreakImpulse || sqrtf(lenSqS(ang)) > j.angBreakImpulse) : 0u;
		return;
	}
	for(int i = 0; i < j.count; i++)
	{
		const SolverRow& c = j.rows[size_t(i)];
		if(c.flags & S_OUTPUT_FORCE)
		{
			lin = add(lin, scale(c.lin0, c.appliedForce));
			ang = add(ang, scale(add(c.ang0, cross(c.lin0, j.rA)), c.appliedForce));
		}
	}
	ang = sub(ang, cross(j.body0WorldOffset, lin));
	force[0] = lin.x; force[1] = lin.y; force[2] = lin.z;
	force[3] = ang.x; force[4] = ang.y; force[5] = ang.z;
	*broken = j.breakable ? uint32_t(sqrtf(lenSqS(lin)) > j.linBreakImpulse || sqrtf(lenSqS(ang)) > j.angBreakImpulse) : 0u;
}
} // namespace

// Same argument layout as the reference harness's pxref_joint_frame.
OX uint32_t orc_joint_frame(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const uint32_t* jointA,
                            const uint32_t* jointB, uint32_t nbJoints, const uint32_t* rowStart, const uint32_t* rowCount, const void* rows,
                            const float* params, const float* gravity, float dt, uint32_t nbPos, uint32_t nbVel, uint32_t batchJoints, float* outVel,
                            float* outPose, uint32_t* outHeaderStart, uint32_t* outHeaderStride, uint32_t* outHeaderType, uint32_t* outOrder,
                            float* outForce, uint32_t* outBroken)
{
	std::vector<BodyVel> vels;
	std::vector<BodyTx> txs;
	std::vector<BodyData> datas;
	std::vector<Tr> poses;
	buildSolverBodies(rigid, nbDyn, staticPose, nbStatic, gravity, dt, vels, txs, datas, poses);
	uint32_t nbRowsTotal = 0;
	for(uint32_t j = 0; j < nbJoints; j++) nbRowsTotal = std::max(nbRowsTotal, rowStart[j] + rowCount[j]);
	std::vector<Row1D> rowCopy(nbRowsTotal ? nbRowsTotal : 1);
	if(nbRowsTotal) memcpy(rowCopy.data(), rows, sizeof(Row1D) * nbRowsTotal);

	BatchOut batch;
	if(batchJoints)
		batchSolverConstraints(jointA, jointB, int(nbJoints), int(nbDyn), batch);
	else
		for(uint32_t i = 0; i < nbJoints; i++)
		{
			batch.order.push_back(int(i));
			batch.headerStart.push_back(i);
			batch.headerStride.push_back(1);
		}
	const uint32_t nbHeaders = uint32_t(batch.headerStart.size());
	for(uint32_t i = 0; i < nbJoints; i++) outOrder[i] = uint32_t(batch.order[i]);

	const float invDt = 1.0f / dt;
	const float stepDt = dt / float(nbPos);
	const float invStepDt = invDt * float(nbPos);
	// PxCreateJointConstraintsTGS(dt = stepDt, totalDt = dt, invDt = invStepDt, invTotalDt = invDt, lengthScale = 1)
	const float biasCoefficient = 2.0f * sqrtf(stepDt / dt);
	std::vector<JointRows> joints(nbJoints);
	for(uint32_t h = 0; h < nbHeaders; h++)
	{
		const uint32_t s0 = batch.headerStart[h], stride = batch.headerStride[h];
		bool block = stride == 4;
		for(uint32_t l = 0; l < stride && block; l++)
			if(rowCount[batch.order[s0 + l]] == 0) block = false;
		outHeaderStart[h] = s0;
		outHeaderStride[h] = stride;
		outHeaderType[h] = block ? TYPE_BLOCK_1D : TYPE_RB_1D;
		for(uint32_t l = 0; l < stride; l++)
		{
			const int ji = batch.order[s0 + l];
			JointIn in;
			in.a = int(jointA[ji]);
			in.b = int(jointB[ji]);
			in.v0 = &vels[in.a]; in.v1 = &vels[in.b];
			in.t0 = &txs[in.a]; in.t1 = &txs[in.b];
			in.d0 = &datas[in.a]; in.d1 = &datas[in.b];
			in.frame0 = poses[in.a];
			in.frame1 = poses[in.b];
			in.params = params + 20 * size_t(ji);
			in.rows = rowCopy.data() + rowStart[ji];
			in.numRows = int(rowCount[ji]);
			setupJoint(in, block, stepDt, dt, invStepDt, invDt, 1.0f, biasCoefficient, joints[ji]);
		}
	}
	float elapsed = 0.0f;
	for(uint32_t it = 0; it < nbPos; it++)
	{
		for(uint32_t k = 0; k < nbJoints; k++)
		{
			JointRows& j = joints[batch.order[k]];
			if(j.block) solveJointBlock(j, vels.data(), txs.data(), elapsed);
			else solveJoint(j, vels.data(), txs.data(), elapsed);
			if(it + 1 == nbPos) concludeJoint(j);
		}
		for(uint32_t b = 0; b < nbDyn; b++) integrateSolverBody(vels[b], txs[b], stepDt);
		elapsed += stepDt;
	}
	for(uint32_t it = 0; it < nbVel; it++)
		for(uint32_t k = 0; k < nbJoints; k++)
		{
			JointRows& j = joints[batch.order[k]];
			if(j.block) solveJointBlock(j, vels.data(), txs.data(), elapsed);
			else solveJoint(j, vels.data(), txs.data(), elapsed);
		}
	for(uint32_t j = 0; j < nbJoints; j++) writeBackJoint(joints[j], outForce + 6 * size_t(j), outBroken + j);
	finishSolverBodies(vels, txs, poses, nbDyn, outVel, outPose);
	return nbHeaders;
}
