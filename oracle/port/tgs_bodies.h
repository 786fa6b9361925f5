// ORACLE (test infrastructure): solver bodies, batching and integration of the
// TGS immediate-mode path (tgs.cpp), shared with the joint path (joint.cpp).
#pragma once
#include "pxmath.h"
#include <stdint.h>
#include <vector>

namespace orc
{
struct RigidBodyData   // PxRigidBodyData, 96 bytes
{
	float linVel[3]; float invMass;
	float angVel[3]; float maxDepenetrationVelocity;
	float invInertia[3]; float maxContactImpulse;
	float q[4]; float p[3];
	float linearDamping, angularDamping, maxLinearVelocitySq, maxAngularVelocitySq;
	uint32_t pad;
};
static_assert(sizeof(RigidBodyData) == 96, "PxRigidBodyData layout");

struct BodyVel      // PxTGSSolverBodyVel fields used by the solver
{
	V3 lin, ang, dLin, dAng;
	float maxAngVel;
	bool kinematic;
};
struct BodyTx       // PxTGSSolverBodyTxInertia
{
	Q dq; V3 p; M33 sqrtInvInertia;
};
struct BodyData     // PxTGSSolverBodyData
{
	V3 origLin, origAng;
	float maxContactImpulse, penBiasClamp, invMass;
};

struct BatchOut
{
	std::vector<int> order;              // ordered constraint indices
	std::vector<uint32_t> headerStart, headerStride;
};

// PxConstructSolverBodiesTGS for nbDyn PxRigidBodyData records, then
// PxConstructStaticSolverBodyTGS for nbStatic poses (7 floats each); arrays
// hold nbDyn + nbStatic bodies, statics last.
void buildSolverBodies(const void* rigid, uint32_t nbDyn, const float* staticPose, uint32_t nbStatic, const float* gravity, float dt,
                       std::vector<BodyVel>& vels, std::vector<BodyTx>& txs, std::vector<BodyData>& datas, std::vector<Tr>& poses);
// PxBatchConstraintsTGS over constraints joining bodyA[i], bodyB[i] (indices >= nbDyn: static).
void batchSolverConstraints(const uint32_t* bodyA, const uint32_t* bodyB, int n, int nbDyn, BatchOut& out);
// integrateCoreStep (DyTGSDynamics.cpp:1403)
void integrateSolverBody(BodyVel& v, BodyTx& t, float dt);
// PxIntegrateSolverBodiesTGS for the first nbDyn bodies: velocities (6 floats,
// world angular) and poses (7 floats).
void finishSolverBodies(const std::vector<BodyVel>& vels, const std::vector<BodyTx>& txs, const std::vector<Tr>& poses, uint32_t nbDyn,
                        float* outVel, float* outPose);
} // namespace orc
