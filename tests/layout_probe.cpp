// Layout probe of the immediate-mode types: prints sizeof / offsetof as JSON.
// Built against the reference's headers (-DPROBE_REFERENCE, by
// tests/golden/make_layouts.py) or against include/gbpx_immediate.h (by
// tests/test_immediate_layout.py); the two tables must agree.
#ifdef PROBE_REFERENCE
#include "PxImmediateMode.h"
#include "geometry/PxSphereGeometry.h"
#include "geometry/PxCapsuleGeometry.h"
#include "geometry/PxBoxGeometry.h"
#include "geometry/PxPlaneGeometry.h"
#include "geometry/PxConvexCoreGeometry.h"
#include "geomutils/PxContactPoint.h"
#include "collision/PxCollisionDefs.h"
#include "solver/PxSolverDefs.h"
using namespace physx;
using namespace physx::immediate;
#else
#include "gbpx_immediate.h"
using namespace gbpx_px;
#endif
#include <cstdio>
#include <cstddef>
#include <cstring>
#define S(T) printf("\"%s\": %zu,\n", #T, sizeof(T))
#define O(T, f) printf("\"%s.%s\": %zu,\n", #T, #f, offsetof(T, f))
int main(){
 printf("{\n");
 S(PxTransform); S(PxGeometry); S(PxSphereGeometry); S(PxCapsuleGeometry); S(PxBoxGeometry); S(PxPlaneGeometry);
 O(PxSphereGeometry, radius); O(PxCapsuleGeometry, radius); O(PxCapsuleGeometry, halfHeight); O(PxBoxGeometry, halfExtents);
 S(PxConvexCoreGeometry);
#ifdef PROBE_REFERENCE
 {
	// the members are private: locate them in a geometry with known values
	const PxConvexCoreGeometry g(PxConvexCore::Cylinder(1.5f, 0.25f), 0.125f);
	const char* b = reinterpret_cast<const char*>(&g);
	const size_t core = static_cast<const char*>(g.getCoreData()) - b;
	size_t type = 0, margin = 0;
	for(size_t o = 8; o + 4 <= sizeof(g); o += 4)
	{
		float f; int i;
		memcpy(&f, b + o, 4); memcpy(&i, b + o, 4);
		if(o < core && i == int(PxConvexCore::eCYLINDER)) type = o;
		if(o >= core + PxConvexCoreGeometry::MAX_CORE_SIZE && f == 0.125f) margin = o;
	}
	printf("\"PxConvexCoreGeometry.mCoreType\": %zu,\n\"PxConvexCoreGeometry.mCore\": %zu,\n\"PxConvexCoreGeometry.mMargin\": %zu,\n", type, core, margin);
 }
#else
 O(PxConvexCoreGeometry, mCoreType); O(PxConvexCoreGeometry, mCore); O(PxConvexCoreGeometry, mMargin);
#endif
 S(PxContactPoint); O(PxContactPoint, normal); O(PxContactPoint, separation); O(PxContactPoint, point); O(PxContactPoint, maxImpulse);
 O(PxContactPoint, targetVel); O(PxContactPoint, staticFriction); O(PxContactPoint, materialFlags); O(PxContactPoint, internalFaceIndex1);
 O(PxContactPoint, dynamicFriction); O(PxContactPoint, restitution); O(PxContactPoint, damping);
 S(PxCache); O(PxCache, mCachedData); O(PxCache, mCachedSize); O(PxCache, mPairData); O(PxCache, mManifoldFlags);
 S(PxRigidBodyData); O(PxRigidBodyData, invMass); O(PxRigidBodyData, angularVelocity); O(PxRigidBodyData, body2World); O(PxRigidBodyData, pad);
 S(PxTGSSolverBodyVel); O(PxTGSSolverBodyVel, angularVelocity); O(PxTGSSolverBodyVel, partitionMask); O(PxTGSSolverBodyVel, deltaAngDt);
 O(PxTGSSolverBodyVel, maxAngVel); O(PxTGSSolverBodyVel, deltaLinDt); O(PxTGSSolverBodyVel, lockFlags); O(PxTGSSolverBodyVel, isKinematic);
 S(PxTGSSolverBodyTxInertia); O(PxTGSSolverBodyTxInertia, body2WorldP); O(PxTGSSolverBodyTxInertia, sqrtInvInertia);
 S(PxTGSSolverBodyData); O(PxTGSSolverBodyData, maxContactImpulse); O(PxTGSSolverBodyData, originalAngularVelocity); O(PxTGSSolverBodyData, penBiasClamp);
 O(PxTGSSolverBodyData, invMass); O(PxTGSSolverBodyData, nodeIndex); O(PxTGSSolverBodyData, reportThreshold);
 S(PxConstraintBatchHeader); O(PxConstraintBatchHeader, stride); O(PxConstraintBatchHeader, constraintType);
 S(PxSolverBody); O(PxSolverBody, maxSolverNormalProgress); O(PxSolverBody, angularState); O(PxSolverBody, solverProgress);
 S(PxSolverBodyData); O(PxSolverBodyData, invMass); O(PxSolverBodyData, angularVelocity); O(PxSolverBodyData, reportThreshold);
 O(PxSolverBodyData, sqrtInvInertia); O(PxSolverBodyData, penBiasClamp); O(PxSolverBodyData, nodeIndex); O(PxSolverBodyData, maxContactImpulse);
 O(PxSolverBodyData, body2World);
 S(PxSolverContactDesc); O(PxSolverContactDesc, desc); O(PxSolverContactDesc, body0); O(PxSolverContactDesc, data0); O(PxSolverContactDesc, data1);
 O(PxSolverContactDesc, bodyFrame0); O(PxSolverContactDesc, bodyFrame1); O(PxSolverContactDesc, bodyState0); O(PxSolverContactDesc, bodyState1);
 O(PxSolverContactDesc, shapeInteraction); O(PxSolverContactDesc, frictionPtr); O(PxSolverContactDesc, contacts); O(PxSolverContactDesc, numContacts);
 O(PxSolverContactDesc, frictionCount); O(PxSolverContactDesc, hasMaxImpulse); O(PxSolverContactDesc, restDistance);
 O(PxSolverContactDesc, maxCCDSeparation); O(PxSolverContactDesc, contactForces); O(PxSolverContactDesc, numContactPatches);
 O(PxSolverContactDesc, axisConstraintCount); O(PxSolverContactDesc, offsetSlop); O(PxSolverConstraintDesc, bodyA); O(PxSolverConstraintDesc, bodyB);
 S(PxSolverConstraintDesc); O(PxSolverConstraintDesc, tgsBodyA); O(PxSolverConstraintDesc, tgsBodyB); O(PxSolverConstraintDesc, bodyADataIndex);
 O(PxSolverConstraintDesc, bodyBDataIndex); O(PxSolverConstraintDesc, linkIndexA); O(PxSolverConstraintDesc, linkIndexB); O(PxSolverConstraintDesc, constraint);
 O(PxSolverConstraintDesc, writeBack); O(PxSolverConstraintDesc, writeBackFriction); O(PxSolverConstraintDesc, progressA); O(PxSolverConstraintDesc, progressB);
 O(PxSolverConstraintDesc, constraintLengthOver16);
 S(PxConstraintInvMassScale);
 S(PxImmediateConstraint); O(PxImmediateConstraint, prep); O(PxImmediateConstraint, constantBlock);
 S(PxTGSSolverContactDesc); O(PxTGSSolverContactDesc, invMassScales); O(PxTGSSolverContactDesc, desc); O(PxTGSSolverContactDesc, body0); O(PxTGSSolverContactDesc, body1);
 O(PxTGSSolverContactDesc, body0TxI); O(PxTGSSolverContactDesc, body1TxI); O(PxTGSSolverContactDesc, bodyData0); O(PxTGSSolverContactDesc, bodyData1);
 O(PxTGSSolverContactDesc, bodyFrame0); O(PxTGSSolverContactDesc, bodyFrame1); O(PxTGSSolverContactDesc, bodyState0); O(PxTGSSolverContactDesc, bodyState1);
 O(PxTGSSolverContactDesc, shapeInteraction); O(PxTGSSolverContactDesc, frictionPtr); O(PxTGSSolverContactDesc, contacts); O(PxTGSSolverContactDesc, numContacts);
 O(PxTGSSolverContactDesc, frictionCount); O(PxTGSSolverContactDesc, hasMaxImpulse); O(PxTGSSolverContactDesc, disableStrongFriction); O(PxTGSSolverContactDesc, hasForceThresholds);
 O(PxTGSSolverContactDesc, restDistance); O(PxTGSSolverContactDesc, maxCCDSeparation); O(PxTGSSolverContactDesc, contactForces); O(PxTGSSolverContactDesc, startFrictionPatchIndex);
 O(PxTGSSolverContactDesc, numFrictionPatches); O(PxTGSSolverContactDesc, startContactPatchIndex); O(PxTGSSolverContactDesc, numContactPatches);
 O(PxTGSSolverContactDesc, axisConstraintCount); O(PxTGSSolverContactDesc, maxImpulse); O(PxTGSSolverContactDesc, torsionalPatchRadius);
 O(PxTGSSolverContactDesc, minTorsionalPatchRadius); O(PxTGSSolverContactDesc, offsetSlop);
 S(Px1DConstraint); O(Px1DConstraint, geometricError); O(Px1DConstraint, angular0); O(Px1DConstraint, velocityTarget); O(Px1DConstraint, linear1);
 O(Px1DConstraint, minImpulse); O(Px1DConstraint, angular1); O(Px1DConstraint, maxImpulse); O(Px1DConstraint, mods); O(Px1DConstraint, flags);
 O(Px1DConstraint, solveHint);
 S(PxTGSSolverConstraintPrepDesc); O(PxTGSSolverConstraintPrepDesc, invMassScales); O(PxTGSSolverConstraintPrepDesc, desc);
 O(PxTGSSolverConstraintPrepDesc, body0); O(PxTGSSolverConstraintPrepDesc, body1); O(PxTGSSolverConstraintPrepDesc, body0TxI);
 O(PxTGSSolverConstraintPrepDesc, body1TxI); O(PxTGSSolverConstraintPrepDesc, bodyData0); O(PxTGSSolverConstraintPrepDesc, bodyData1);
 O(PxTGSSolverConstraintPrepDesc, bodyFrame0); O(PxTGSSolverConstraintPrepDesc, bodyFrame1); O(PxTGSSolverConstraintPrepDesc, bodyState0);
 O(PxTGSSolverConstraintPrepDesc, bodyState1); O(PxTGSSolverConstraintPrepDesc, writeback); O(PxTGSSolverConstraintPrepDesc, rows);
 O(PxTGSSolverConstraintPrepDesc, numRows); O(PxTGSSolverConstraintPrepDesc, linBreakForce); O(PxTGSSolverConstraintPrepDesc, angBreakForce);
 O(PxTGSSolverConstraintPrepDesc, minResponseThreshold); O(PxTGSSolverConstraintPrepDesc, disablePreprocessing);
 O(PxTGSSolverConstraintPrepDesc, improvedSlerp); O(PxTGSSolverConstraintPrepDesc, driveLimitsAreForces); O(PxTGSSolverConstraintPrepDesc, extendedLimits);
 O(PxTGSSolverConstraintPrepDesc, disableConstraint); O(PxTGSSolverConstraintPrepDesc, body0WorldOffset); O(PxTGSSolverConstraintPrepDesc, cA2w);
 O(PxTGSSolverConstraintPrepDesc, cB2w);
 printf("\"end\": 0\n}\n");
 return 0;
}
