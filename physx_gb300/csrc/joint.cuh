// Joints (1D constraints) of the TGS immediate-mode path on the GB300:
//   PxCreateJointConstraintsTGS (physx/source/immediatemode/src/NpImmediateMode.cpp:1480)
//     per-pair path: setupSolverConstraintStep (lowleveldynamics/src/DyTGSContactPrep.cpp:1939)
//       with preprocessRows / orthogonalize (lowleveldynamics/src/DyConstraintSetup.cpp:492,213)
//     4-wide path (a header of stride 4 whose joints all have rows):
//       setupSolverConstraintStep4 (lowleveldynamics/src/DyTGSContactPrepBlock.cpp:1719)
//   PxSolveConstraintsTGS: solve1DStep (DyTGSContactPrep.cpp:2418) / solve1DStep4
//     (DyTGSContactPrepBlock.cpp:2957), conclude1DStep (:2750), writeBack1DStep (:2837)
//     / writeBack1D4 (DyTGSContactPrepBlock.cpp:3418)
// Rigid bodies only.  A joint is one JointRecord (header + up to 12 rows); a
// lane of a 4-wide header keeps its own record and is solved with that path's
// operation order (its padding rows apply no impulse and are not stored).
// Arithmetic follows the reference's operation order; the translation units
// that include this header are compiled without fused multiply-add.
#pragma once
#include "solver.cuh"

namespace gbpx
{
namespace joint
{
using namespace tgs;

// Px1DConstraint (physx/include/PxConstraintDesc.h:194), 80 bytes: the caller's row
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

constexpr int MAX_ROWS = 12;   // Dy::MAX_CONSTRAINT_ROWS
// Px1DConstraintFlag and PxConstraintSolveHint values
constexpr uint32_t F_SPRING = 1, F_ACCEL_SPRING = 2, F_RESTITUTION = 4, F_KEEPBIAS = 8, F_OUTPUT_FORCE = 16, F_HAS_DRIVE_LIMIT = 32, F_ANGULAR = 64;
constexpr uint32_t H_EQUALITY = 2048, H_INEQUALITY = 2049, H_ROT_EQUALITY = 1024, H_ROT_INEQUALITY = 1025;
// solver row flags (lowleveldynamics/src/DySolverConstraintTypes.h:60)
constexpr uint32_t S_OUTPUT_FORCE = 2, S_KEEP_BIAS = 4, S_ROT_EQ = 8, S_ORTHO_TARGET = 16, S_SPRING = 32, S_INEQUALITY = 64, S_ACCEL_SPRING = 128;
// PxConstraintBatchHeader::constraintType of joint headers (DY_SC_TYPE_RB_1D / _BLOCK_1D)
constexpr uint32_t TYPE_RB_1D = 2, TYPE_BLOCK_1D = 8;
// per-joint parameters (20 floats): invMassScales (linear0, angular0, linear1,
// angular1), cA2w, cB2w, body0WorldOffset, linBreakForce, angBreakForce,
// minResponseThreshold, flags (float of PARAM_* bits), 3 unused
constexpr int PARAM_FLOATS = 20;
constexpr uint32_t PARAM_DISABLE_PREPROCESSING = 1, PARAM_IMPROVED_SLERP = 2, PARAM_DRIVE_LIMITS_ARE_FORCES = 4;

// SolverConstraint1DStep, 96 bytes
struct __align__(16) JointRow
{
	V3 lin0; float error;
	V3 lin1; float biasScale;
	V3 ang0; float velMultiplier;
	V3 ang1; float velTarget;
	float minImpulse, maxImpulse, appliedForce, maxBias;
	uint32_t flags;
	float angularErrorScale;   // 1: angular row (angular motion counts in the error), 0: linear
	float pad[2];
};
static_assert(sizeof(JointRow) == 96, "joint row layout");

// SolverConstraint1DHeaderStep + rows, 1344 bytes
struct __align__(16) JointRecord
{
	uint32_t bodyA, bodyB;
	uint32_t count;     // rows in use
	uint32_t flags;     // JR_BLOCK: a lane of a 4-wide header; JR_BREAKABLE
	float invMass0, invMass1, angScale0, angScale1;   // angScale1: -angular1 (per-pair), +angular1 (4-wide)
	float linBreakImpulse, angBreakImpulse, pad0, pad1;
	V3 body0WorldOffset; float pad2;
	V3 rA; float pad3;
	V3 rB; float pad4;
	V3 orthoAxis0[3];
	V3 orthoAxis1[3];
	float orthoRecipResponse[3], orthoError[3];
	JointRow rows[MAX_ROWS];
};
constexpr uint32_t JR_BLOCK = 1, JR_BREAKABLE = 2;
static_assert(sizeof(JointRecord) == 1344, "joint record layout");
// the immediate-mode entry points store a record as its header and the rows in use
static_assert(offsetof(JointRecord, rows) == 192 && offsetof(JointRecord, count) == 8, "joint record header layout");

// ---------------------------------------------------------------- the 4-wide path's sums
// V4MulAdd chains sum x + (y + z) (V4Dot3, DyTGSContactPrepBlock.cpp:2952);
// QuatRotate4's dot and the transposed inertia product sum (x + y) + z.
__device__ __forceinline__ float dotX_YZ(V3 a, V3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ float dotXY_Z(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 m33TMulXY_Z(const M33& m, V3 v) { return v3(dotXY_Z(m.c0, v), dotXY_Z(m.c1, v), dotXY_Z(m.c2, v)); }
// QuatRotate4 (DyTGSContactPrepBlock.cpp:57): 2 (v (w^2 - 1/2) + (u x v) w + u (u.v))
__device__ __forceinline__ V3 qRotate4(Q q, V3 v)
{
	const float w2 = q.w * q.w + (-0.5f);
	const V3 u = v3(q.x, q.y, q.z);
	const V3 temp = add(scale(cross(u, v), q.w), scale(v, w2));
	return scale(add(scale(u, dotXY_Z(u, v)), temp), 2.0f);
}

struct F4 { float x, y, z, w; };
__device__ __forceinline__ F4 f4(float x, float y, float z, float w) { F4 r = {x, y, z, w}; return r; }
__device__ __forceinline__ F4 f4NegScaleSub(F4 a, F4 b, float t) { return f4(a.x - b.x * t, a.y - b.y * t, a.z - b.z * t, a.w - b.w * t); }

// ---------------------------------------------------------------- row preprocessing
// orthogonalize (DyConstraintSetup.cpp:213): Gram-Schmidt over the mass metric;
// the geometric error rides in linear0's W lane and the velocity target in
// angular0's, equality rows become the base vectors of the later rows.
__device__ __forceinline__ void orthogonalize(Row1D* rows, const int* idx, F4* angSqrt0, F4* angSqrt1, int rowCount, int eqRowCount, float im0,
                                              float im1, float is0, float is1)
{
	F4 lin0m[6], ang0m[6], lin0AndG[6], ang0AndT[6];
	V3 lin1m[6], ang1m[6], lin1[6], ang1[6];
	for(int i = 0; i < rowCount; i++)
	{
		Row1D& r = rows[idx[i]];
		F4 l0AndG = f4(r.linear0[0], r.linear0[1], r.linear0[2], r.geometricError);
		F4 a0AndT = f4(r.angular0[0], r.angular0[1], r.angular0[2], r.velocityTarget);
		V3 l1 = v3(r.linear1[0], r.linear1[1], r.linear1[2]);
		V3 a1 = v3(r.angular1[0], r.angular1[1], r.angular1[2]);
		F4 aL0 = angSqrt0[i], aL1 = angSqrt1[i];
		const int elim = i < eqRowCount ? i : eqRowCount;
		for(int j = 0; j < elim; j++)
		{
			const V3 s0 = v3(l1.x * lin1m[j].x + l0AndG.x * lin0m[j].x, l1.y * lin1m[j].y + l0AndG.y * lin0m[j].y,
			                 l1.z * lin1m[j].z + l0AndG.z * lin0m[j].z);
			const V3 s1 = v3(aL1.x * ang1m[j].x + aL0.x * ang0m[j].x, aL1.y * ang1m[j].y + aL0.y * ang0m[j].y,
			                 aL1.z * ang1m[j].z + aL0.z * ang0m[j].z);
			const float t = sumElems(add(s0, s1));
			l0AndG = f4NegScaleSub(l0AndG, lin0AndG[j], t);
			a0AndT = f4NegScaleSub(a0AndT, ang0AndT[j], t);
			l1 = sub(l1, scale(lin1[j], t));
			a1 = sub(a1, scale(ang1[j], t));
			aL0 = f4NegScaleSub(aL0, angSqrt0[j], t);
			aL1 = f4NegScaleSub(aL1, angSqrt1[j], t);
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
			const V3 l0m = scale(l0, im0);
			const V3 l1m = scale(l1, im1);
			const F4 a0m = f4(aL0.x * is0, aL0.y * is0, aL0.z * is0, aL0.w * is0);
			const F4 a1m = f4(aL1.x * is1, aL1.y * is1, aL1.z * is1, aL1.w * is1);
			const V3 s0 = v3(l0.x * l0m.x + l1.x * l1m.x, l0.y * l0m.y + l1.y * l1m.y, l0.z * l0m.z + l1.z * l1m.z);
			const V3 s1 = v3(a0m.x * aL0.x + a1m.x * aL1.x, a0m.y * aL0.y + a1m.y * aL1.y, a0m.z * aL0.z + a1m.z * aL1.z);
			const float s = sumElems(add(s0, s1));
			const float a = s > 0.0f ? 1.0f / s : 0.0f;
			lin0m[i] = f4(l0m.x * a, l0m.y * a, l0m.z * a, 0.0f);
			ang0m[i] = f4(a0m.x * a, a0m.y * a, a0m.z * a, 0.0f);
			lin1m[i] = scale(l1m, a);
			ang1m[i] = scale(v3(a1m.x, a1m.y, a1m.z), a);
		}
	}
}

// ---------------------------------------------------------------- row constants (DyCpuGpu1dConstraint.h)
__device__ __forceinline__ float bounceVelocity(uint32_t flags, float jointSpeed, float threshold, float restitution, float geometricError)
{
	const float bounceVel = jointSpeed * (-restitution);
	if((flags & F_RESTITUTION) && (-jointSpeed > threshold) && ((bounceVel * geometricError) <= 0.0f)) return bounceVel;
	return 0.0f;
}

__device__ __forceinline__ float maxBiasVelocity(uint32_t flags, float jointSpeed, float threshold, float restitution, float geometricError,
                                                 float lengthScale, float recipSimDt)
{
	if(flags & F_SPRING) return FLT_MAX;
	if(bounceVelocity(flags, jointSpeed, threshold, restitution, geometricError) != 0.0f) return 0.0f;
	if(flags & F_ANGULAR) return recipSimDt * 0.75f;
	return recipSimDt * 15.0f * lengthScale;
}

// compute1dConstraintSolverConstantsTGS (:423): biasScale, error, velMultiplier, velTarget
__device__ __forceinline__ void solverConstants(const Row1D& c, float jointSpeed, float initJointSpeed, float unitResponse, float recipUnitResponse,
                                                float erp, float stepDt, float recipStepDt, JointRow& s)
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

__device__ __forceinline__ uint32_t internalFlags(uint32_t flags, uint32_t hint)
{
	uint32_t f = 0;
	if(flags & F_SPRING) f |= S_SPRING;
	if(flags & F_ACCEL_SPRING) f |= S_ACCEL_SPRING;
	if(flags & F_OUTPUT_FORCE) f |= S_OUTPUT_FORCE;
	if(flags & F_KEEPBIAS) f |= S_KEEP_BIAS;
	if(hint & 1u) f |= S_INEQUALITY;
	return f;
}

struct PrepTimes { float stepDt, simDt, recipStepDt, recipSimDt, lengthScale, biasCoefficient; };

// One joint's record (setupSolverConstraintStep, or one lane of
// setupSolverConstraintStep4 when block): rows are the caller's, rewritten as
// the reference rewrites them (solve hints of angular rows, orthogonalisation).
__device__ __forceinline__ void prepJoint(Row1D* rows, int numRows, const float* params, bool block, const BodyVel& v0, const BodyVel& v1,
                                          const BodyTx& t0, const BodyTx& t1, const BodyData& d0, const BodyData& d1, V3 frame0P, V3 frame1P,
                                          const PrepTimes& pt, JointRecord& out)
{
	const float ims0 = params[0], ims1 = params[1], ims2 = params[2], ims3 = params[3];
	const uint32_t pflags = uint32_t(params[16]);
	const bool disablePre = (pflags & PARAM_DISABLE_PREPROCESSING) != 0, limitsAreForces = (pflags & PARAM_DRIVE_LIMITS_ARE_FORCES) != 0;
	out.count = uint32_t(numRows);
	out.flags = (block ? JR_BLOCK : 0u) | ((params[13] != FLT_MAX || params[14] != FLT_MAX) ? JR_BREAKABLE : 0u);
	out.invMass0 = d0.invMass * ims0;
	out.invMass1 = d1.invMass * ims2;
	out.angScale0 = ims1;
	out.angScale1 = block ? ims3 : -ims3;
	out.linBreakImpulse = params[13] * pt.simDt;
	out.angBreakImpulse = params[14] * pt.simDt;
	out.body0WorldOffset = v3(params[10], params[11], params[12]);
	out.rA = sub(v3(params[4], params[5], params[6]), frame0P);
	out.rB = sub(v3(params[7], params[8], params[9]), frame1P);
	for(int k = 0; k < 3; k++)
	{
		out.orthoAxis0[k] = out.orthoAxis1[k] = v3(0.0f, 0.0f, 0.0f);
		out.orthoRecipResponse[k] = out.orthoError[k] = 0.0f;
	}
	if(numRows <= 0) return;
	for(int i = 0; i < numRows; i++)
	{
		Row1D& r = rows[i];
		if(r.flags & F_ANGULAR)
		{
			if(r.solveHint == H_EQUALITY) r.solveHint = uint16_t(H_ROT_EQUALITY);
			else if(r.solveHint == H_INEQUALITY) r.solveHint = uint16_t(H_ROT_INEQUALITY);
		}
	}
	// preprocessRows: stable insertion sort by solve hint, I^(-1/2) * angular,
	// orthogonalisation of the equality groups (hint >> 8 == 4 rotational, == 8 linear)
	int idx[MAX_ROWS];
	for(int i = 0; i < numRows; i++)
	{
		int j = i;
		for(; j > 0 && rows[i].solveHint < rows[idx[j - 1]].solveHint; j--) idx[j] = idx[j - 1];
		idx[j] = i;
	}
	F4 angSqrt0[MAX_ROWS], angSqrt1[MAX_ROWS];
	for(int i = 0; i < numRows; i++)
	{
		const Row1D& r = rows[idx[i]];
		const V3 a0 = m33MulV(t0.sqrtInvInertia, v3(r.angular0[0], r.angular0[1], r.angular0[2]));
		const V3 a1 = m33MulV(t1.sqrtInvInertia, v3(r.angular1[0], r.angular1[1], r.angular1[2]));
		angSqrt0[i] = f4(a0.x, a0.y, a0.z, 0.0f);
		angSqrt1[i] = f4(a1.x, a1.y, a1.z, 0.0f);
	}
	if(!disablePre)
	{
		for(int i = 0; i < numRows;)
		{
			const uint32_t group = uint32_t(rows[idx[i]].solveHint) >> 8;
			const int start = i++;
			while(i < numRows && (uint32_t(rows[idx[i]].solveHint) >> 8) == group) i++;
			if(group == 4 || group == 8)
			{
				int bCount = start;
				for(; bCount < i && (rows[idx[bCount]].solveHint & 255) == 0; bCount++)
					;
				orthogonalize(rows, idx + start, angSqrt0 + start, angSqrt1 + start, i - start, bCount - start, d0.invMass * ims0,
				              d1.invMass * ims2, ims1, ims3);
			}
		}
	}
	const float erp = 0.5f * pt.biasCoefficient;
	int orthoCount = 0;
	for(int i = 0; i < numRows; i++)
	{
		const Row1D& c = rows[idx[i]];
		JointRow& s = out.rows[i];
		const float driveScale = ((c.flags & F_HAS_DRIVE_LIMIT) && limitsAreForces) ? pt.simDt : 1.0f;
		s.lin0 = v3(c.linear0[0], c.linear0[1], c.linear0[2]);
		s.lin1 = v3(c.linear1[0], c.linear1[1], c.linear1[2]);
		s.ang0 = v3(c.angular0[0], c.angular0[1], c.angular0[2]);
		s.ang1 = v3(c.angular1[0], c.angular1[1], c.angular1[2]);
		s.minImpulse = c.minImpulse * driveScale;
		s.maxImpulse = c.maxImpulse * driveScale;
		s.appliedForce = 0.0f;
		s.angularErrorScale = 1.0f;
		s.pad[0] = s.pad[1] = 0.0f;
		const V3 aS0 = v3(angSqrt0[i].x, angSqrt0[i].y, angSqrt0[i].z), aS1 = v3(angSqrt1[i].x, angSqrt1[i].y, angSqrt1[i].z);
		float unitResponse, vel0, vel1;
		if(!block)
		{
			const float linSumMass = lenSqS(s.lin0) * d0.invMass * ims0 + lenSqS(s.lin1) * d1.invMass * ims2;
			unitResponse = lenSqS(aS0) * ims1 + lenSqS(aS1) * ims3 + linSumMass;
			vel0 = dotS(d0.origLin, s.lin0) + dotS(d0.origAng, s.ang0);
			vel1 = dotS(d1.origLin, s.lin1) + dotS(d1.origAng, s.ang1);
		}
		else
		{
			// setupSolverConstraintStep4 (DyTGSContactPrepBlock.cpp:2087-2106): pre-scaled
			// masses, per-body sums, body B's speed taken along I^(-1/2) angular1
			unitResponse = (lenSqS(s.lin0) * out.invMass0 + lenSqS(aS0) * ims1) + (lenSqS(s.lin1) * out.invMass1 + lenSqS(aS1) * ims3);
			vel0 = dotX_YZ(s.lin0, d0.origLin) + dotX_YZ(s.ang0, d0.origAng);
			vel1 = dotX_YZ(s.lin1, d1.origLin) + dotX_YZ(aS1, d1.origAng);
		}
		float initJointSpeed = 0.0f;
		if(v0.kinematic) initJointSpeed -= vel0;
		if(v1.kinematic) initJointSpeed += vel1;
		const float jointSpeed = vel0 - vel1;
		if(!(c.flags & F_ANGULAR))
		{
			s.ang0 = v3(0.0f, 0.0f, 0.0f);
			s.ang1 = v3(0.0f, 0.0f, 0.0f);
			s.angularErrorScale = 0.0f;
		}
		const float recipUnitResponse = unitResponse <= params[15] ? 0.0f : 1.0f / unitResponse;
		s.maxBias = maxBiasVelocity(c.flags, jointSpeed, c.mod1, c.mod0, c.geometricError, pt.lengthScale, pt.recipSimDt);
		solverConstants(c, jointSpeed, initJointSpeed, unitResponse, recipUnitResponse, erp, pt.stepDt, pt.recipStepDt, s);
		s.flags = internalFlags(c.flags, c.solveHint);
		if(!disablePre)
		{
			if(c.solveHint == H_ROT_EQUALITY)
			{
				s.flags |= S_ROT_EQ;
				out.orthoAxis0[orthoCount] = scale(aS0, ims1);
				out.orthoAxis1[orthoCount] = scale(aS1, ims3);
				out.orthoRecipResponse[orthoCount] = recipUnitResponse;
				out.orthoError[orthoCount] = c.geometricError;
				orthoCount++;
			}
			else if(c.solveHint & H_EQUALITY)
				s.flags |= S_ORTHO_TARGET;
		}
	}
}

// ---------------------------------------------------------------- solve
// solve1DStep (DyTGSContactPrep.cpp:2418) on bodies b0, b1
__device__ __forceinline__ void solveJointPair(JointRecord& j, BodyVel& b0, BodyVel& b1, const BodyTx& t0, const BodyTx& t1, float elapsed)
{
	V3 linVel0 = b0.lin, linVel1 = b1.lin, angState0 = b0.ang, angState1 = b1.ang;
	const V3 ra = qRotate(t0.dq, j.rA), rb = qRotate(t1.dq, j.rB);
	const V3 ang0 = b0.dAng, ang1 = b1.dAng;
	const V3 raMotion = sub(add(ra, b0.dLin), j.rA);
	const V3 rbMotion = sub(add(rb, b1.dLin), j.rB);
	float orthoErr[3];
	for(int k = 0; k < 3; k++) orthoErr[k] = j.orthoError[k] + (dotA(j.orthoAxis0[k], ang0) - dotA(j.orthoAxis1[k], ang1));
	const uint32_t count = j.count;
	for(uint32_t i = 0; i < count; i++)
	{
		JointRow& c = j.rows[i];
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
			error = error - c.biasScale * (orthoErr[0] * proj[0] + (orthoErr[1] * proj[1] + orthoErr[2] * proj[2]));
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
		const V3 va = add(mul(linVel0, c.lin0), mul(angState0, raXnI));
		const V3 vb = add(mul(linVel1, c.lin1), mul(angState1, rbXnI));
		const float normalVel = sumElems(sub(va, vb));
		const float clamped = fclamp(c.appliedForce + (vMul * normalVel + constant), c.minImpulse, c.maxImpulse);
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

// one lane of solve1DStep4 (DyTGSContactPrepBlock.cpp:2957)
__device__ __forceinline__ void solveJointBlock(JointRecord& j, BodyVel& b0, BodyVel& b1, const BodyTx& t0, const BodyTx& t1, float elapsed)
{
	V3 linVel0 = b0.lin, linVel1 = b1.lin, angState0 = b0.ang, angState1 = b1.ang;
	const V3 ra = qRotate4(t0.dq, j.rA), rb = qRotate4(t1.dq, j.rB);
	const V3 dAng0 = b0.dAng, dAng1 = b1.dAng;
	const V3 raMotion = sub(add(ra, b0.dLin), j.rA);
	const V3 rbMotion = sub(add(rb, b1.dLin), j.rB);
	float orthoErr[3];
	for(int k = 0; k < 3; k++) orthoErr[k] = j.orthoError[k] + (dotX_YZ(j.orthoAxis0[k], dAng0) - dotX_YZ(j.orthoAxis1[k], dAng1));
	const float mass0 = j.invMass0, mass1 = j.invMass1, scale0 = j.angScale0, scale1 = j.angScale1;
	const uint32_t count = j.count;
	for(uint32_t i = 0; i < count; i++)
	{
		JointRow& c = j.rows[i];
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
			err = err - c.biasScale * (orthoErr[0] * proj[0] + (orthoErr[1] * proj[1] + orthoErr[2] * proj[2])) * coef;
		}
		const bool spring = (c.flags & S_SPRING) != 0;
		const float deltaAng = c.angularErrorScale * (dotX_YZ(d0, dAng0) - dotX_YZ(d1, dAng1));
		const float deltaLin = dotX_YZ(c.lin0, raMotion) - dotX_YZ(c.lin1, rbMotion);
		const float motion = deltaLin + deltaAng;
		const float errorChange = spring ? motion : motion - c.velTarget * elapsed;
		const float response = (mass0 * dotX_YZ(c.lin0, c.lin0) + scale0 * dotX_YZ(d0, d0)) + (mass1 * dotX_YZ(c.lin1, c.lin1) + scale1 * dotX_YZ(d1, d1));
		const float recipResponse = response > 0.0f ? 1.0f / response : 0.0f;
		const float vMul = spring ? c.velMultiplier : recipResponse * c.velMultiplier;
		const float minBias = -((c.flags & S_INEQUALITY) ? FLT_MAX : c.maxBias);
		const float bias = fclamp(errorChange * c.biasScale + err, minBias, c.maxBias);
		const float constant = spring ? bias + c.velTarget : recipResponse * (bias + c.velTarget);
		const float normalVel = (dotX_YZ(c.lin0, linVel0) - dotX_YZ(c.lin1, linVel1)) + (dotX_YZ(d0, angState0) - dotX_YZ(d1, angState1));
		const float clamped = fclamp(c.appliedForce + (vMul * normalVel + constant), c.minImpulse, c.maxImpulse);
		const float deltaF = clamped - c.appliedForce;
		c.appliedForce = clamped;
		linVel0 = add(scale(c.lin0, deltaF * mass0), linVel0);
		linVel1 = sub(linVel1, scale(c.lin1, deltaF * mass1));
		angState0 = add(scale(d0, deltaF * scale0), angState0);
		angState1 = sub(angState1, scale(d1, deltaF * scale1));
	}
	b0.lin = linVel0; b0.ang = angState0;
	b1.lin = linVel1; b1.ang = angState1;
}

__device__ __forceinline__ void solveJoint(JointRecord& j, BodyVel& b0, BodyVel& b1, const BodyTx& t0, const BodyTx& t1, float elapsed)
{
	if(j.count == 0) return;
	if(j.flags & JR_BLOCK) solveJointBlock(j, b0, b1, t0, t1, elapsed);
	else solveJointPair(j, b0, b1, t0, t1, elapsed);
}

// conclude1DStep (DyTGSContactPrep.cpp:2750): after the last position iteration
__device__ __forceinline__ void concludeJoint(JointRecord& j)
{
	for(uint32_t i = 0; i < j.count; i++)
	{
		JointRow& c = j.rows[i];
		if(!(c.flags & S_KEEP_BIAS)) { c.biasScale = 0.0f; c.error = 0.0f; }
		if(c.flags & S_SPRING) { c.velMultiplier = 0.0f; c.biasScale = 0.0f; c.error = 0.0f; c.velTarget = 0.0f; }
	}
}

// writeBack1DStep / writeBack1D4: linear and angular impulse of the rows that
// output force (6 floats) and the broken flag
__device__ __forceinline__ void writeBackJoint(const JointRecord& j, float* force, uint32_t* broken)
{
	V3 lin = v3(0.0f, 0.0f, 0.0f), ang = v3(0.0f, 0.0f, 0.0f);
	if(j.flags & JR_BLOCK)
	{
		// the 4-wide write-back takes the angular part from angular0 alone and
		// forms its body0WorldOffset term as that code does
		for(uint32_t i = 0; i < j.count; i++)
		{
			const JointRow& c = j.rows[i];
			const float f = (c.flags & S_OUTPUT_FORCE) ? c.appliedForce : 0.0f;
			lin = add(scale(c.lin0, f), lin);
			ang = add(scale(c.ang0, f), ang);
		}
		const V3 o = j.body0WorldOffset;
		ang = v3(ang.x - (o.y * lin.z - o.x * lin.y), ang.y - (o.z * lin.x - o.y * lin.z), ang.z - (o.x * lin.y - o.z * lin.x));
	}
	else
	{
		for(uint32_t i = 0; i < j.count; i++)
		{
			const JointRow& c = j.rows[i];
			if(c.flags & S_OUTPUT_FORCE)
			{
				lin = add(lin, scale(c.lin0, c.appliedForce));
				ang = add(ang, scale(add(c.ang0, cross(c.lin0, j.rA)), c.appliedForce));
			}
		}
		ang = sub(ang, cross(j.body0WorldOffset, lin));
	}
	force[0] = lin.x; force[1] = lin.y; force[2] = lin.z;
	force[3] = ang.x; force[4] = ang.y; force[5] = ang.z;
	*broken = (j.flags & JR_BREAKABLE) ? uint32_t(sqrtf(lenSqS(lin)) > j.linBreakImpulse || sqrtf(lenSqS(ang)) > j.angBreakImpulse) : 0u;
}
} // namespace joint
} // namespace gbpx
